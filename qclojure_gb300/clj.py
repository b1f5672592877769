"""The few Clojure runtime behaviours that show in the reference's outputs.

A Clojure map of more than eight entries iterates in the order of its hash trie, so
wherever the reference walks such a map (to emit operations, sum floats, or break ties
in a stable sort) the order follows the keys' hashes. Printing a lazy sequence with
`str` gives the class name and the Java hash code instead of its elements. This module
restates those rules from Clojure's published runtime semantics (Murmur3 `hasheq`,
Java `hashCode`) so host code can produce the same orders and strings.
"""
from __future__ import annotations

M32 = 0xFFFFFFFF
_GOLDEN = 0x9E3779B9


def _rotl(v: int, r: int) -> int:
    return ((v << r) | (v >> (32 - r))) & M32


def _mix_k1(k: int) -> int:
    return (_rotl((k * 0xCC9E2D51) & M32, 15) * 0x1B873593) & M32


def _mix_h1(h: int, k: int) -> int:
    return (_rotl(h ^ k, 13) * 5 + 0xE6546B64) & M32


def _fmix(h: int, length: int) -> int:
    h ^= length
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & M32
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & M32
    return h ^ (h >> 16)


def _signed(v: int) -> int:
    v &= M32
    return v - (1 << 32) if v & 0x80000000 else v


def hash_long(x: int) -> int:
    """`hash` of a long: Murmur3 over its two 32-bit halves (unsigned 32-bit result)."""
    if x == 0:
        return 0
    x &= 0xFFFFFFFFFFFFFFFF
    h = _mix_h1(_mix_h1(0, _mix_k1(x & M32)), _mix_k1(x >> 32))
    return _fmix(h, 8)


def _hash_unencoded_chars(s: str) -> int:
    units = s.encode("utf-16-le")
    chars = [units[i] | (units[i + 1] << 8) for i in range(0, len(units), 2)]
    h = 0
    for i in range(1, len(chars), 2):
        h = _mix_h1(h, _mix_k1(chars[i - 1] | (chars[i] << 16)))
    if len(chars) & 1:
        h ^= _mix_k1(chars[-1])
    return _fmix(h, 2 * len(chars))


def _hash_combine(seed: int, h: int) -> int:
    """Util.hashCombine on Java ints: seed ^ (h + golden + (seed << 6) + (seed >> 2))."""
    seed, h = _signed(seed), _signed(h)
    return (seed ^ _signed(h + _GOLDEN + _signed(seed << 6) + (seed >> 2))) & M32


def hash_keyword(name: str) -> int:
    """`hash` of an unqualified keyword :name (unsigned 32-bit)."""
    return (_hash_combine(_hash_unencoded_chars(name), 0) + _GOLDEN) & M32


def java_string_hash(s: str) -> int:
    h = 0
    units = s.encode("utf-16-le")
    for i in range(0, len(units), 2):
        h = (31 * h + (units[i] | (units[i + 1] << 8))) & M32
    return h


def keyword_hash_code(name: str) -> int:
    """Java hashCode of an unqualified keyword (unsigned 32-bit)."""
    return (_hash_combine(java_string_hash(name), 0) + _GOLDEN) & M32


def map_order(keys: list, hasheq) -> list:
    """The order in which a map built by `into {}` / `assoc` from these keys (in this
    insertion order) yields them: insertion order up to 8 entries (an array map), else
    the hash trie's order, which visits keys by the 5-bit digits of their hash, lowest
    digit first."""
    if len(keys) <= 8:
        return list(keys)

    def digits(k):
        h = hasheq(k)
        return tuple((h >> s) & 31 for s in range(0, 32, 5))

    return sorted(keys, key=digits)


def lazy_seq_of_keywords_str(names: list[str]) -> str:
    """`(str s)` for a lazy sequence of keywords: the class name, '@' and the Java hash
    code in hex, where the hash code is 31-polynomial over the elements' hash codes (an
    empty sequence hashes to 1)."""
    h = 1
    for n in names:
        h = (31 * h + keyword_hash_code(n)) & M32
    return f"clojure.lang.LazySeq@{h:x}"
