"""Generate the golden fixtures under tests/golden from the UNMODIFIED reference.

Runs only where the reference source tree exists (it builds oracle/_ref with
``make -C oracle ref``).  The fixtures it writes are committed, so the tests
never need the reference at run time.

    python tests/golden/make_golden.py --ref-root <reference checkout>   (or QT_REF_TREE=<checkout>)

Fixtures:
  gates.json      every gate tensor the reference's Node classes build (src/Node.h:197-898)
  pairs.json      ContractIndices (src/Network.h:876-971) on seeded random operands
  networks.json   sample circuits: a recorded stochastic ordering (mCreatedFrom walk,
                  preprocess.h:41-46), the reference's value and flop count for it,
                  and the same ordering replayed through ContractGivenSequence
  qaoa.json       light-cone QASM text of the MaxCut term generator (src/maxcut.h:105-233)
  linegraph.json  wire numbering of the LineGraph constructor (src/LineGraph.h:92-171)
  config1.json    seeded 6-qubit depth-10 Rx + CZ circuits, <Z_0>: this build's seeded
                  stochastic ordering recorded, the reference's value and flop count for
                  it (ContractGivenSequence, ContractionTools.h:392-411)
"""
import argparse
import hashlib
import json
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "qt_ref_harness")


def canon_bytes(arr):
    """float64 bytes with -0.0 folded into +0.0."""
    a = np.asarray(arr, dtype=np.complex128).view(np.float64) + 0.0
    return a.tobytes()


def digest(arr):
    return hashlib.sha256(canon_bytes(arr)).hexdigest()


def run(args, cwd):
    r = subprocess.run([HARNESS] + args, capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError(f"harness {args} failed rc={r.returncode}: {r.stdout[-400:]} {r.stderr[-400:]}")
    return r.stdout


def parse_kv(out):
    d = {}
    for line in out.splitlines():
        p = line.split()
        if p:
            d.setdefault(p[0], []).append(p[1:])
    return d


def pair_operands(seed, ra, rb, ns):
    """Seeded operands + index maps for one pair case (regenerated by the tests)."""
    rng = np.random.default_rng(seed)
    sa = [int(x) for x in rng.permutation(ra)[:ns]]
    sb = [int(x) for x in rng.permutation(rb)[:ns]]
    fa = [i for i in range(ra) if i not in sa]
    fb = [i for i in range(rb) if i not in sb]
    a = rng.standard_normal(4 ** ra) + 1j * rng.standard_normal(4 ** ra)
    b = rng.standard_normal(4 ** rb) + 1j * rng.standard_normal(4 ** rb)
    return a, b, [1] * len(fa) + [0] * len(fb), fa + fb, sa, sb


def gen_pairs(cwd):
    cases = []
    shapes = [(0, 0, 0), (1, 1, 1), (2, 1, 1), (1, 2, 1), (2, 2, 1), (2, 2, 2), (4, 2, 1), (2, 4, 1), (4, 4, 1),
              (4, 4, 2), (4, 4, 3), (4, 4, 4), (5, 3, 2), (3, 5, 2), (6, 2, 1), (6, 4, 2), (5, 5, 1), (5, 5, 3),
              (7, 2, 1), (3, 3, 3), (6, 6, 1), (6, 6, 4), (8, 2, 1), (2, 8, 1), (7, 7, 5)]
    for n, (ra, rb, ns) in enumerate(shapes):
        seed = 1000 + n
        a, b, ffa, fi, sa, sb = pair_operands(seed, ra, rb, ns)
        buf = struct.pack("<iii", ra, rb, len(fi))
        for x, y in zip(ffa, fi):
            buf += struct.pack("<ii", x, y)
        buf += struct.pack("<i", len(sa))
        for x, y in zip(sa, sb):
            buf += struct.pack("<ii", x, y)
        buf += a.astype(np.complex128).tobytes() + b.astype(np.complex128).tobytes()
        pin, pout = "/tmp/qt_golden_pair_in.bin", "/tmp/qt_golden_pair_out.bin"
        with open(pin, "wb") as f:
            f.write(buf)
        run(["pair", pin, pout], cwd)
        c = np.frombuffer(open(pout, "rb").read(), dtype=np.complex128)
        case = {"seed": seed, "rank_a": ra, "rank_b": rb, "n_sum": ns, "free_from_a": ffa, "free_idx": fi,
                "sum_a": sa, "sum_b": sb, "sha256": digest(c)}
        if c.size <= 256:
            case["c"] = [[float(v.real), float(v.imag)] for v in c]
        cases.append(case)
    return cases


def gen_gates(cwd):
    out = run(["gates", "Samples/arbitrary2qubitmatrixset"], cwd)
    gates = []
    for line in out.splitlines():
        p = line.split()
        name, rank = p[1], int(p[2])
        vals = [float(x) for x in p[3:]]
        gates.append({"name": name, "rank": rank, "values": [[vals[2 * i], vals[2 * i + 1]] for i in range(len(vals) // 2)]})
    return gates


# (circuit, measurement text) pairs; the circuit text is embedded in the fixture
NETWORK_CASES = [
    ("rand-nq6-cn2-d10_rx.qasm", "Z T T T T T"),
    ("rand-nq6-cn2-d10_rx.qasm", "Y T Y T Y T Y T"),
    ("rand-nq6-cn2-d10_rxz.qasm", "Z T Z T Z T Z T"),
    ("rand-nq6-cn2-d10_rxyz.qasm", "X T X T X T X T"),
    ("rand-nq6-cn2-d10_rxyz.qasm", "Z T Z T Z T Z T"),
    ("test_JW.qasm", "Z T T T"),
    ("test_JW.qasm", "Y X X Y"),
    ("qft8.qasm", None),
    ("qft4.qasm", "X Y Z 0"),
    ("bell_pair.qasm", "0 0"),
    ("bell_pair.qasm", "1 1"),
    ("4regRand20Node1-p1.qasm", "@measure125.txt"),
    ("tofolli.qasm", "1 1 T"),
    ("catStateEightQubits.qasm", "Z Z T T T T T T"),
    ("teleportation.qasm", "Z T X"),
    ("control_phase.qasm", "X Y"),
    ("swap.qasm", "Z X"),
    ("rotationRz.qasm", "X"),
    ("hadamard.qasm", "0"),
]


def gen_networks(ref_root, cwd):
    nets = []
    for k, (qasm, meas) in enumerate(NETWORK_CASES):
        qpath = os.path.join("Samples", qasm)
        qtext = open(os.path.join(ref_root, qpath)).read()
        if meas is None:
            mtext = open(os.path.join(ref_root, "Samples", "measureSampleOne.txt")).read()
        elif meas.startswith("@"):
            mtext = open(os.path.join(ref_root, "Samples", meas[1:])).read()
        else:
            mtext = meas
        mpath = f"/tmp/qt_golden_meas_{k}.txt"
        with open(mpath, "w") as f:
            f.write(mtext)
        d = parse_kv(run(["stoch", qpath, mpath, "1"], cwd))
        if "exception" in d:
            raise RuntimeError(f"{qasm}: {d['exception']}")
        seq = [int(x) for x in d["sequence"][0]]
        pairs = [[seq[i], seq[i + 1]] for i in range(0, len(seq), 2)]
        spath = f"/tmp/qt_golden_seq_{k}.txt"
        with open(spath, "w") as f:
            f.write("\n".join(f"{a} {b}" for a, b in pairs) + "\n")
        r = parse_kv(run(["seq", qpath, mpath, spath], cwd))
        # arbitrary gate files named by def1/def2 lines travel with the fixture
        gate_files = {}
        for line in qtext.splitlines():
            t = line.split(" ")
            if t and t[0] in ("def1", "def2") and len(t) >= 3:
                gate_files[t[2]] = open(os.path.join(ref_root, t[2])).read()
        nets.append({
            "name": qasm, "qasm": qtext, "measure": mtext, "gate_files": gate_files,
            "sequence": pairs,
            "value": [float(d["value"][0][0]), float(d["value"][0][1])],
            "flops": int(d["flops"][0][0]),
            "replay_value": [float(r["value"][0][0]), float(r["value"][0][1])],
        })
    return nets


def gen_qaoa(ref_root, cwd):
    out = []
    for dgf, p, bg in (("4regRand30Node26.dgf", 1, [0.3, 0.7]), ("3regRand30Node50.dgf", 2, [0.3, 0.1, 0.7, 0.45]),
                       ("3regRand30Node50.dgf", 1, [0.125, 2.9])):
        text = run(["qaoa", os.path.join("Samples", dgf), str(p)] + [repr(x) for x in bg], cwd)
        terms, cur, head = [], None, None
        for line in text.splitlines(keepends=True):
            if line.startswith("term "):
                cur, head = [], line.split()
                continue
            if line.startswith("endterm"):
                terms.append({"edge": [int(head[2]), int(head[3])], "qubits": int(head[4]), "qasm": "".join(cur)})
                continue
            cur.append(line)
        out.append({"dgf_name": dgf, "dgf": open(os.path.join(ref_root, "Samples", dgf)).read(), "p": p,
                    "betas_gammas": bg, "terms": terms})
    return out


def gen_linegraph(ref_root, cwd):
    out = []
    for qasm, meas in (("bell_pair.qasm", "Z Z"), ("rand-nq6-cn2-d10_rx.qasm", "Z T T T T T"), ("test_JW.qasm", "Z T T T")):
        mpath = "/tmp/qt_golden_lg_meas.txt"
        with open(mpath, "w") as f:
            f.write(meas)
        text = run(["lgwires", os.path.join("Samples", qasm), mpath], cwd)
        nodes = []
        for line in text.splitlines():
            p = line.split()
            wires = [[int(x) for x in w.split(":")] for w in p[2:]]
            nodes.append({"node": int(p[1]), "wires": wires})
        out.append({"name": qasm, "qasm": open(os.path.join(ref_root, "Samples", qasm)).read(), "measure": meas,
                    "nodes": nodes})
    return out


def gen_reduce(ref_root, cwd):
    """ReduceCircuit's contractions, then a stochastic finish (main.cpp:112 path)."""
    out = []
    for qasm, meas in (("test_JW.qasm", "Z T T T"), ("rand-nq6-cn2-d10_rxyz.qasm", "Z T Z T Z T"),
                       ("qft4.qasm", "X Y Z 0"), ("catStateEightQubits.qasm", "Z Z T T T T T T")):
        mpath = "/tmp/qt_golden_reduce_meas.txt"
        with open(mpath, "w") as f:
            f.write(meas)
        d = parse_kv(run(["reduce", os.path.join("Samples", qasm), mpath], cwd))
        red = [int(x) for x in d["sequence"][0]]
        full = [int(x) for x in d["sequence"][1]]
        out.append({"name": qasm, "qasm": open(os.path.join(ref_root, "Samples", qasm)).read(), "measure": meas,
                    "reduced_nodes": [int(x) for x in d["reduced_nodes"][0]],
                    "reduce_sequence": [[red[i], red[i + 1]] for i in range(0, len(red), 2)],
                    "sequence": [[full[i], full[i + 1]] for i in range(0, len(full), 2)],
                    "value": [float(d["value"][0][0]), float(d["value"][0][1])]})
    return out


CONFIG1_SEEDS = (1, 2, 3, 4, 5)
CONFIG1_MEASURE = "Z T T T T T"   # <Z_0>, the other qubits traced


def gen_config1(cwd):
    sys.path.insert(0, REPO)
    import qtorch_gb300 as qg
    from qtorch_gb300.circuits import config1_circuit_text
    out = []
    for seed in CONFIG1_SEEDS:
        qtext = config1_circuit_text(seed)
        plan = qg.Plan(qtext, CONFIG1_MEASURE, ordering="stochastic", seed=seed, symbolic=True)
        pairs = [list(p) for p in plan.sequence()]
        qpath, mpath, spath = (f"/tmp/qt_golden_c1_{seed}.{x}" for x in ("qasm", "meas", "seq"))
        with open(qpath, "w") as f:
            f.write(qtext)
        with open(mpath, "w") as f:
            f.write(CONFIG1_MEASURE)
        with open(spath, "w") as f:
            f.write("\n".join(f"{a} {b}" for a, b in pairs) + "\n")
        r = parse_kv(run(["seq", qpath, mpath, spath], cwd))
        if "exception" in r:
            raise RuntimeError(f"config 1 seed {seed}: {r['exception']}")
        out.append({"seed": seed, "qasm": qtext, "measure": CONFIG1_MEASURE, "sequence": pairs,
                    "value": [float(r["value"][0][0]), float(r["value"][0][1])], "flops": int(r["flops"][0][0])})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=os.environ.get("QT_REF_TREE"), required="QT_REF_TREE" not in os.environ)
    ap.add_argument("--only", nargs="*", help="regenerate only these fixtures (the stochastic ones change every run)")
    args = ap.parse_args()
    src = os.path.join(args.ref_root, "src")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF_SRC={src}"], check=True)
    cwd = args.ref_root
    makers = {
        "gates.json": lambda: gen_gates(cwd),
        "pairs.json": lambda: gen_pairs(cwd),
        "networks.json": lambda: gen_networks(args.ref_root, cwd),
        "qaoa.json": lambda: gen_qaoa(args.ref_root, cwd),
        "linegraph.json": lambda: gen_linegraph(args.ref_root, cwd),
        "reduce.json": lambda: gen_reduce(args.ref_root, cwd),
        "config1.json": lambda: gen_config1(cwd),
    }
    fixtures = {k: f() for k, f in makers.items() if not args.only or k in args.only}
    for name, data in fixtures.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(data, f, indent=0)
        print(name, len(data), file=sys.stderr)


if __name__ == "__main__":
    main()
