"""Write tests/golden/reference_kat.json: known-answer cases of the reference's tests.

Each case restates one assertion of QClojure's own test suite (file:line under
test/org/soulspace/qclojure/) as data: an initial basis state, the operations
(in the reference's map form) and what the test asserts about the result:

  state_exact   the full state vector equals `expected` exactly (the test uses =)
  state_close   every amplitude within `tol` of `expected`
  amp_close     amplitude `index` within `tol` of `value`
  amp_abs_lt / amp_abs_gt    |amplitude `index`| below / above `value`
  amp_im_eq     imaginary part of amplitude `index` equals `value`
  pauli_eq      <psi|P|psi> of `pauli` equals `value` (tolerance `tol`, 0 = exact)
  ham_eq        sum c_j <P_j> equals `value` (tolerance `tol`)
  obs_close     <psi|O_t|psi> of a 2x2 observable within `tol` of `value`
  var_close     variance <O^2> - <O>^2 within `tol` of `value`
  norm_close    sum |a|^2 within `tol` of 1
  counts_exact  sampled histogram equals `counts` (deterministic outcomes)
  counts_ratio  outcomes only in `allowed`, ratio of `first` in (lo, hi)

Run: python tests/golden/make_reference_kat.py
"""
import json
import math
from pathlib import Path

S2 = 1 / math.sqrt(2)
T = "test/org/soulspace/qclojure/"


def c(re, im=0.0):
    return [re, im]


def basis(n, idx):
    v = [c(0.0) for _ in range(1 << n)]
    v[idx] = c(1.0)
    return v


def op(t, **p):
    d = {"operation-type": t}
    if p:
        d["operation-params"] = {k.replace("_", "-"): v for k, v in p.items()}
    return d


cases = []


def case(name, src, n, init, ops, checks):
    cases.append({"name": name, "source": src, "num-qubits": n, "initial-basis": init, "operations": ops,
                  "checks": checks})


# --- gate_test.clj -----------------------------------------------------------
G = T + "domain/gate_test.clj"
case("X|0>=|1>", G + ":16-24", 1, 0, [op("x", target=0)], [{"kind": "state_exact", "expected": basis(1, 1)}])
case("X|1>=|0>", G + ":16-24", 1, 1, [op("x", target=0)], [{"kind": "state_exact", "expected": basis(1, 0)}])
case("Z|0>=|0>", G + ":26-35", 1, 0, [op("z", target=0)], [{"kind": "state_exact", "expected": basis(1, 0)}])
case("Z|1>=-|1>", G + ":26-35", 1, 1, [op("z", target=0)],
     [{"kind": "state_exact", "expected": [c(0.0), c(-1.0)]}])
for init, exp in ((0, 1), (1, 0)):
    case(f"HZH|{init}>=X|{init}>", G + ":37-49", 1, init, [op("h", target=0), op("z", target=0), op("h", target=0)],
         [{"kind": "state_close", "expected": basis(1, exp), "tol": 1e-10}])
case("H|0>", G + ":52-61", 1, 0, [op("h", target=0)],
     [{"kind": "state_close", "expected": [c(S2), c(S2)], "tol": 1e-10}])
for init in (0, 1):
    case(f"HH|{init}>", G + ":63-73", 1, init, [op("h", target=0), op("h", target=0)],
         [{"kind": "state_close", "expected": basis(1, init), "tol": 1e-10}])
for init, exp in ((0, 0), (1, 1), (2, 3), (3, 2)):
    case(f"CNOT|{init:02b}>", G + ":76-97", 2, init, [op("cnot", control=0, target=1)],
         [{"kind": "state_exact", "expected": basis(2, exp)}])
case("Bell via gates", G + ":100-116", 2, 0, [op("h", target=0), op("cnot", control=0, target=1)],
     [{"kind": "state_close", "expected": [c(S2), c(0), c(0), c(S2)], "tol": 1e-10}])
for init in (0, 1, 2):
    case(f"RydbergCZ|{init:02b}>", G + ":126-145", 2, init, [op("rydberg-cz", control=0, target=1)],
         [{"kind": "state_exact", "expected": basis(2, init)}])
case("RydbergCZ|11>", G + ":126-145", 2, 3, [op("rydberg-cz", control=0, target=1)],
     [{"kind": "amp_close", "index": 3, "value": c(-1.0), "tol": 0.0}])
case("RydbergCPhase|00>", G + ":147-160", 2, 0, [op("rydberg-cphase", control=0, target=1, angle=math.pi / 4)],
     [{"kind": "state_exact", "expected": basis(2, 0)}])
case("RydbergCPhase|11>", G + ":147-160", 2, 3, [op("rydberg-cphase", control=0, target=1, angle=math.pi / 4)],
     [{"kind": "amp_close", "index": 3, "value": c(math.cos(math.pi / 4), math.sin(math.pi / 4)), "tol": 1e-10}])
case("Blockade|00>", G + ":162-174", 2, 0, [op("rydberg-blockade", qubit_indices=[0, 1], angle=math.pi / 4)],
     [{"kind": "state_exact", "expected": basis(2, 0)}])
case("Blockade|01> changes", G + ":162-174", 2, 1, [op("rydberg-blockade", qubit_indices=[0, 1], angle=math.pi / 4)],
     [{"kind": "amp_close", "index": 1, "value": c(math.cos(math.pi / 4), math.sin(math.pi / 4)), "tol": 1e-10}])
case("GlobalX|000>", G + ":177-183", 3, 0, [op("global-x")],
     [{"kind": "amp_abs_close", "index": 7, "value": 1.0, "tol": 1e-10}])
case("GlobalH|00>", G + ":185-193", 2, 0, [op("global-h")],
     [{"kind": "amp_abs_close", "index": i, "value": 0.5, "tol": 1e-10} for i in range(4)])
case("GlobalRZ|00>", G + ":195-206", 2, 0, [op("global-rz", angle=math.pi / 4)],
     [{"kind": "amp_abs_close", "index": 0, "value": 1.0, "tol": 1e-10}])
case("GlobalRX|00> moves", G + ":195-206", 2, 0, [op("global-rx", angle=math.pi / 4)],
     [{"kind": "amp_abs_lt", "index": 0, "value": 0.99}])
case("GlobalRY|00> moves", G + ":195-206", 2, 0, [op("global-ry", angle=math.pi / 4)],
     [{"kind": "amp_abs_lt", "index": 0, "value": 0.99}])
case("SWAP|01>", G + ":209-219", 2, 1, [op("swap", qubit1=0, qubit2=1)],
     [{"kind": "state_exact", "expected": basis(2, 2)}])
case("SWAP|10>", G + ":209-219", 2, 2, [op("swap", qubit1=0, qubit2=1)],
     [{"kind": "state_exact", "expected": basis(2, 1)}])
case("iSWAP|01>", G + ":221-230", 2, 1, [op("iswap", qubit1=0, qubit2=1)],
     [{"kind": "amp_im_eq", "index": 2, "value": 1.0}])
case("iSWAP|10>", G + ":221-230", 2, 2, [op("iswap", qubit1=0, qubit2=1)],
     [{"kind": "amp_im_eq", "index": 1, "value": 1.0}])
for init, exp in ((0, 0), (6, 7), (7, 6)):
    case(f"Toffoli|{init:03b}>", G + ":232-248", 3, init, [op("toffoli", control1=0, control2=1, target=2)],
         [{"kind": "state_exact", "expected": basis(3, exp)}])
for init, exp in ((0, 0), (1, 1), (2, 2), (3, 3), (4, 4), (5, 6), (6, 5), (7, 7)):
    case(f"Fredkin|{init:03b}>", G + ":251-272", 3, init, [op("fredkin", control=0, target1=1, target2=2)],
         [{"kind": "state_exact", "expected": basis(3, exp)}])
    case(f"FredkinFredkin|{init:03b}>", G + ":274-280", 3, init,
         [op("fredkin", control=0, target1=1, target2=2), op("fredkin", control=0, target1=1, target2=2)],
         [{"kind": "state_exact", "expected": basis(3, init)}])
case("Y|0>=i|1>", G + ":283-295", 1, 0, [op("y", target=0)],
     [{"kind": "amp_abs_lt", "index": 0, "value": 1e-10}, {"kind": "amp_close", "index": 1, "value": c(0, 1), "tol": 1e-10}])
case("Y|1>=-i|0>", G + ":283-295", 1, 1, [op("y", target=0)],
     [{"kind": "amp_close", "index": 0, "value": c(0, -1), "tol": 1e-10}, {"kind": "amp_abs_lt", "index": 1, "value": 1e-10}])
for init in (0, 1):
    case(f"YY|{init}>", G + ":297-308", 1, init, [op("y", target=0), op("y", target=0)],
         [{"kind": "state_close", "expected": basis(1, init), "tol": 1e-10}])
# controlled Y is reached through :controlled (circuit.clj:889-931)
cy = lambda: op("controlled", control_qubits=[0], target_gate="y", target_qubits=[1])  # noqa: E731
for init in (0, 1):
    case(f"CY|{init:02b}>", G + ":311-328", 2, init, [cy()], [{"kind": "state_exact", "expected": basis(2, init)}])
case("CY|10>", G + ":311-328", 2, 2, [cy()],
     [{"kind": "amp_abs_lt", "index": 2, "value": 1e-10}, {"kind": "amp_abs_gt", "index": 3, "value": 0.9}])
case("CY|11>", G + ":311-328", 2, 3, [cy()],
     [{"kind": "amp_abs_gt", "index": 2, "value": 0.9}, {"kind": "amp_abs_lt", "index": 3, "value": 1e-10}])
for init in (0, 1, 2):
    case(f"CZ|{init:02b}>", G + ":330-350", 2, init, [op("cz", control=0, target=1)],
         [{"kind": "state_exact", "expected": basis(2, init)}])
case("CZ|11>", G + ":330-350", 2, 3, [op("cz", control=0, target=1)],
     [{"kind": "amp_close", "index": 3, "value": c(-1.0), "tol": 1e-10}])
case("S|0>", G + ":353-363", 1, 0, [op("s", target=0)], [{"kind": "state_exact", "expected": basis(1, 0)}])
case("S|1>=i|1>", G + ":353-363", 1, 1, [op("s", target=0)],
     [{"kind": "amp_close", "index": 1, "value": c(0, 1), "tol": 0.0}])
case("T|0>", G + ":365-376", 1, 0, [op("t", target=0)], [{"kind": "state_exact", "expected": basis(1, 0)}])
case("T|1>", G + ":365-376", 1, 1, [op("t", target=0)],
     [{"kind": "amp_close", "index": 1, "value": c(math.sqrt(2) / 2, math.sqrt(2) / 2), "tol": 1e-10}])
case("SdagS|1>", G + ":378-390", 1, 1, [op("s", target=0), op("s-dag", target=0)],
     [{"kind": "amp_close", "index": 1, "value": c(1.0), "tol": 1e-10}])
case("TdagT|1>", G + ":378-390", 1, 1, [op("t", target=0), op("t-dag", target=0)],
     [{"kind": "amp_close", "index": 1, "value": c(1.0), "tol": 1e-10}])
case("RX(pi/2)|0>", G + ":393-403", 1, 0, [op("rx", target=0, angle=math.pi / 2)],
     [{"kind": "state_close", "expected": [c(S2), c(0, -S2)], "tol": 1e-10}])
case("RY(pi/2)|0>", G + ":405-415", 1, 0, [op("ry", target=0, angle=math.pi / 2)],
     [{"kind": "state_close", "expected": [c(S2), c(S2)], "tol": 1e-10}])
case("RZ(pi/2)|0>", G + ":417-431", 1, 0, [op("rz", target=0, angle=math.pi / 2)],
     [{"kind": "amp_close", "index": 0, "value": c(math.sqrt(2) / 2, -math.sqrt(2) / 2), "tol": 1e-10}])
case("RZ(pi/2)|1>", G + ":417-431", 1, 1, [op("rz", target=0, angle=math.pi / 2)],
     [{"kind": "amp_close", "index": 1, "value": c(math.sqrt(2) / 2, math.sqrt(2) / 2), "tol": 1e-10}])
for g in ("crx", "cry"):
    case(f"{g}|00>", G + ":434-455", 2, 0, [op(g, control=0, target=1, angle=math.pi / 2)],
         [{"kind": "state_exact", "expected": basis(2, 0)}])
    case(f"{g}|10> moves", G + ":434-455", 2, 2, [op(g, control=0, target=1, angle=math.pi / 2)],
         [{"kind": "amp_abs_lt", "index": 2, "value": 0.99}])
case("normalization preserved", G + ":457-528", 3, 5,
     [op("h", target=0), op("rx", target=1, angle=0.7), op("cnot", control=0, target=2),
      op("rydberg-blockade", qubit_indices=[0, 1, 2], angle=0.3), op("fredkin", control=2, target1=0, target2=1),
      op("global-ry", angle=1.1)],
     [{"kind": "norm_close", "tol": 1e-10}])

# --- circuit_test.clj ----------------------------------------------------------
case("Bell circuit", T + "domain/circuit_test.clj:410-427", 2, 0,
     [op("h", target=0), op("cnot", control=0, target=1)],
     [{"kind": "state_close", "expected": [c(S2), c(0), c(0), c(S2)], "tol": 1e-10}])

# --- result_test.clj / hamiltonian_test.clj --------------------------------------
R = T + "domain/result_test.clj"
PZ = [[c(1), c(0)], [c(0), c(-1)]]
PX = [[c(0), c(1)], [c(1), c(0)]]
case("<Z>|0>", R + ":47-55", 1, 0, [], [{"kind": "obs_close", "observable": PZ, "target": 0, "value": 1.0, "tol": 1e-10}])
case("<X>|+>", R + ":57-62", 1, 0, [op("h", target=0)],
     [{"kind": "obs_close", "observable": PX, "target": 0, "value": 1.0, "tol": 1e-10},
      {"kind": "obs_close", "observable": PZ, "target": 0, "value": 0.0, "tol": 1e-10}])
case("Var Z|0>", R + ":71-79", 1, 0, [], [{"kind": "var_close", "observable": PZ, "target": 0, "value": 0.0, "tol": 1e-10}])
case("Var Z|+>", R + ":81-87", 1, 0, [op("h", target=0)],
     [{"kind": "var_close", "observable": PZ, "target": 0, "value": 1.0, "tol": 1e-10}])
case("H=Z on |0>", R + ":90-97", 1, 0, [], [{"kind": "ham_eq", "terms": [[1.0, "Z"]], "value": 1.0, "tol": 1e-10}])
case("H=0.5Z+0.5X on |+>", R + ":99-104", 1, 0, [op("h", target=0)],
     [{"kind": "ham_eq", "terms": [[0.5, "Z"], [0.5, "X"]], "value": 0.5, "tol": 1e-10}])
H = T + "domain/hamiltonian_test.clj"
case("<Z>|0>=1 exact", H + ":66-72", 1, 0, [], [{"kind": "pauli_eq", "pauli": "Z", "value": 1.0, "tol": 0.0}])
case("<Z>|1>=-1 exact", H + ":66-72", 1, 1, [], [{"kind": "pauli_eq", "pauli": "Z", "value": -1.0, "tol": 0.0}])
case("<Z>|+>~0", H + ":66-72", 1, 0, [op("h", target=0)], [{"kind": "pauli_eq", "pauli": "Z", "value": 0.0, "tol": 1e-10}])
case("<X>|0>~0", H + ":74-78", 1, 0, [], [{"kind": "pauli_eq", "pauli": "X", "value": 0.0, "tol": 1e-10}])
case("<X>|1>~0", H + ":74-78", 1, 1, [], [{"kind": "pauli_eq", "pauli": "X", "value": 0.0, "tol": 1e-10}])
case("<X>|+>=1", H + ":74-78", 1, 0, [op("h", target=0)], [{"kind": "pauli_eq", "pauli": "X", "value": 1.0, "tol": 1e-10}])
case("<X>|->=-1", H + ":74-78", 1, 1, [op("h", target=0)], [{"kind": "pauli_eq", "pauli": "X", "value": -1.0, "tol": 1e-10}])
for init in (0, 1):
    case(f"<I>|{init}>=1", H + ":80-84", 1, init, [], [{"kind": "pauli_eq", "pauli": "I", "value": 1.0, "tol": 1e-10}])
case("<I>|+>=1", H + ":80-84", 1, 0, [op("h", target=0)], [{"kind": "pauli_eq", "pauli": "I", "value": 1.0, "tol": 1e-10}])
case("<ZZ>|00>=1", H + ":86-94", 2, 0, [], [{"kind": "pauli_eq", "pauli": "ZZ", "value": 1.0, "tol": 0.0},
                                             {"kind": "pauli_eq", "pauli": "II", "value": 1.0, "tol": 0.0},
                                             {"kind": "pauli_eq", "pauli": "ZI", "value": 1.0, "tol": 0.0}])
case("<ZZ>|11>=1", H + ":86-94", 2, 3, [], [{"kind": "pauli_eq", "pauli": "ZZ", "value": 1.0, "tol": 0.0}])
case("2I+Z on |0> = 3", H + ":98-104", 1, 0, [], [{"kind": "ham_eq", "terms": [[2.0, "I"], [1.0, "Z"]], "value": 3.0, "tol": 0.0}])
case("2I+Z on |1> = 1", H + ":98-104", 1, 1, [], [{"kind": "ham_eq", "terms": [[2.0, "I"], [1.0, "Z"]], "value": 1.0, "tol": 0.0}])
case("multi-term = 1.4", H + ":106-115", 2, 0, [],
     [{"kind": "ham_eq", "terms": [[1.0, "II"], [0.5, "ZI"], [-0.3, "IZ"], [0.2, "ZZ"]],
       "value": 1.0 + 0.5 + -0.3 + 0.2, "tol": 0.0}])

# --- ideal_simulator_test.clj (backend-level, sampled) ----------------------------
I = T + "adapter/backend/ideal_simulator_test.clj"
case("X then measure: 100 x 1", I + ":157-171", 1, 0, [op("x", target=0)],
     [{"kind": "counts_exact", "shots": 100, "counts": {"1": 100}}])
case("X, CNOT: 100 x 3", I + ":172-185", 2, 0, [op("x", target=0), op("cnot", control=0, target=1)],
     [{"kind": "counts_exact", "shots": 100, "counts": {"3": 100}}])
case("H: ratio in (0.40, 0.60)", I + ":103-118", 1, 0, [op("h", target=0)],
     [{"kind": "counts_ratio", "shots": 1000, "allowed": [0, 1], "first": 0, "lo": 0.40, "hi": 0.60}])
case("Bell: ratio in (0.45, 0.55)", I + ":119-136", 2, 0, [op("h", target=0), op("cnot", control=0, target=1)],
     [{"kind": "counts_ratio", "shots": 1000, "allowed": [0, 3], "first": 0, "lo": 0.45, "hi": 0.55}])
case("GHZ3: ratio in (0.45, 0.55)", I + ":137-155", 3, 0,
     [op("h", target=0), op("cnot", control=0, target=1), op("cnot", control=1, target=2)],
     [{"kind": "counts_ratio", "shots": 1000, "allowed": [0, 7], "first": 0, "lo": 0.45, "hi": 0.55}])

# --- measurement_test.clj (collapse) ----------------------------------------------
M = T + "domain/measurement_test.clj"
case("H then measure leaves one amplitude", M + ":115-128", 1, 0,
     [op("h", target=0), op("measure", measurement_qubits=[0])],
     [{"kind": "nonzero_count", "value": 1}])
case("measure-all leaves one amplitude", M + ":142-153", 2, 0,
     [op("h", target=0), op("h", target=1), op("measure", measurement_qubits=[0, 1])],
     [{"kind": "nonzero_count", "value": 1}, {"kind": "norm_close", "tol": 1e-10}])
case("partial measurement leaves two amplitudes", M + ":173-183", 2, 0,
     [op("h", target=0), op("h", target=1), op("measure", measurement_qubits=[0])],
     [{"kind": "nonzero_count", "value": 2}, {"kind": "norm_close", "tol": 1e-10}])
case("collapsed |+> has magnitude 1", M + ":185-196", 1, 0,
     [op("h", target=0), op("measure", measurement_qubits=[0])],
     [{"kind": "nonzero_count", "value": 1}, {"kind": "max_abs_close", "value": 1.0, "tol": 1e-10}])

out = Path(__file__).with_name("reference_kat.json")
out.write_text(json.dumps({"generator": "tests/golden/make_reference_kat.py", "cases": cases}, indent=1))
print(f"wrote {len(cases)} cases to {out}")
