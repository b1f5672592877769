"""A small EDN reader for the reference's data files (its device catalogue, noise models).

Reads the subset of EDN those files use: maps, vectors, lists, sets, strings, keywords,
integers and floats (with exponents, `N` / `M` suffixes and ratios), `nil`, `true`,
`false`, other symbols, `;` comments, commas as whitespace and `#_` discards. Keywords
become their name without the colon ("all-to-all", "gate-noise"), which is how the
Python mirror spells the reference's keyword keys and values; sets become frozensets
(so a set can hold sets), vectors and lists become lists, maps become dicts.
"""
from __future__ import annotations

import re
from fractions import Fraction

_DELIMS = set("()[]{}\"; \t\r\n,")
_NUMBER = re.compile(r"^[-+]?(\d+)(\.\d*)?([eE][-+]?\d+)?[NM]?$")
_RATIO = re.compile(r"^[-+]?\d+/\d+$")
_ESCAPES = {"n": "\n", "t": "\t", "r": "\r", "\\": "\\", '"': '"', "b": "\b", "f": "\f"}
_CHARS = {"newline": "\n", "space": " ", "tab": "\t", "return": "\r"}


class EdnError(ValueError):
    """Malformed or unsupported EDN."""


class _Reader:
    def __init__(self, text: str):
        self.s, self.i = text, 0

    def _skip(self) -> None:
        s = self.s
        while self.i < len(s):
            c = s[self.i]
            if c in " \t\r\n,":
                self.i += 1
            elif c == ";":
                j = s.find("\n", self.i)
                self.i = len(s) if j < 0 else j + 1
            elif s.startswith("#_", self.i):
                self.i += 2
                self.read()
            else:
                return

    def at_end(self) -> bool:
        self._skip()
        return self.i >= len(self.s)

    def _token(self) -> str:
        j = self.i
        while j < len(self.s) and self.s[j] not in _DELIMS:
            j += 1
        tok, self.i = self.s[self.i:j], j
        return tok

    def _seq(self, close: str) -> list:
        out = []
        while True:
            self._skip()
            if self.i >= len(self.s):
                raise EdnError(f"missing {close!r}")
            if self.s[self.i] == close:
                self.i += 1
                return out
            out.append(self.read())

    def _string(self) -> str:
        out, s = [], self.s
        self.i += 1
        while self.i < len(s):
            c = s[self.i]
            if c == '"':
                self.i += 1
                return "".join(out)
            if c == "\\":
                e = s[self.i + 1:self.i + 2]
                if e == "u":
                    out.append(chr(int(s[self.i + 2:self.i + 6], 16)))
                    self.i += 6
                    continue
                if e not in _ESCAPES:
                    raise EdnError(f"bad escape \\{e}")
                out.append(_ESCAPES[e])
                self.i += 2
                continue
            out.append(c)
            self.i += 1
        raise EdnError("unterminated string")

    def read(self):
        self._skip()
        if self.i >= len(self.s):
            raise EdnError("unexpected end of input")
        c = self.s[self.i]
        if c == "{":
            self.i += 1
            items = self._seq("}")
            if len(items) % 2:
                raise EdnError("a map needs an even number of forms")
            return {_key(items[k]): items[k + 1] for k in range(0, len(items), 2)}
        if c == "[":
            self.i += 1
            return self._seq("]")
        if c == "(":
            self.i += 1
            return self._seq(")")
        if self.s.startswith("#{", self.i):
            self.i += 2
            return frozenset(_key(x) for x in self._seq("}"))
        if c == '"':
            return self._string()
        if c in ")]}":
            raise EdnError(f"unexpected {c!r}")
        if c == "\\":
            self.i += 1
            tok = self._token() or self.s[self.i - 1]
            return _CHARS.get(tok, tok[:1])
        if c == "#":
            raise EdnError("tagged literals are not supported")
        return _atom(self._token())


def _key(v):
    """Map keys and set members must hash: lists become tuples."""
    if isinstance(v, list):
        return tuple(_key(x) for x in v)
    if isinstance(v, dict):
        return tuple(sorted((k, _key(x)) for k, x in v.items()))
    return v


def _atom(tok: str):
    if tok.startswith(":"):
        if len(tok) < 2:
            raise EdnError("empty keyword")
        return tok[1:]
    if tok in ("nil", "true", "false"):
        return {"nil": None, "true": True, "false": False}[tok]
    m = _NUMBER.match(tok)
    if m:
        body = tok.rstrip("NM")
        if m.group(2) is None and m.group(3) is None and not tok.endswith("M"):
            return int(body)
        return float(body)
    if _RATIO.match(tok):
        return float(Fraction(tok))
    if not tok:
        raise EdnError("empty token")
    return tok


def loads(text: str):
    """The single form in `text`."""
    r = _Reader(text)
    v = r.read()
    if not r.at_end():
        raise EdnError("more than one form")
    return v


def load(path: str):
    with open(path, encoding="utf-8") as f:
        return loads(f.read())
