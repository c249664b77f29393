"""Restatement of qTorch's MaxCut QAOA term generator — TEST INFRASTRUCTURE ONLY.

Follows src/maxcut.h:56-103 (ExtraData::ReadInData), :105-186 (PopulateIterations,
PopulateIterationsHelper), :194-233 (outputInitialPlusStateToFile,
applyU_CsThenU_Bs) and src/maxcut.cpp:166-190 (the per-edge QASM/measurement
text written by F_p).  Angles are written with the ostream default format,
6 significant digits (``%g``), exactly as the reference's ``operator<<`` does.
"""


def read_dgf(text):
    """(pairs, num_qubits) from .dgf text: 'c' lines are comments, 'e a b' edges."""
    pairs = []
    mx = 0
    # operator>>(char) reads the first non-space character of a line: 'c' skips
    # the rest of the line, 'e' is followed by two ints, anything else is skipped
    for line in text.splitlines():
        s = line.strip()
        if not s:
            continue
        if s[0] == "c":
            continue
        if s[0] != "e":
            continue
        parts = s[1:].split()
        a, b = int(parts[0]), int(parts[1])
        mx = max(mx, a, b)
        pairs.append((a, b))
    return pairs, mx + 1


def light_cones(pairs, num_qubits, p):
    """(real_iterations, qubits_needed) per edge, as PopulateIterations builds them."""
    adj = [[] for _ in range(num_qubits)]
    for a, b in pairs:
        adj[a].append(b)
        adj[b].append(a)
    real_iters, needed = [], []
    for first, second in pairs:
        mp = [-1] * num_qubits
        working = [first, second]
        mp[first] = 0
        qn = 1
        new_working = [False] * num_qubits
        checked = [False] * num_qubits
        in_working = [False] * num_qubits
        in_working[first] = True
        in_working[second] = True
        iters = []
        for _level in range(p):
            for v in working:
                for t in adj[v]:
                    if not checked[t]:
                        if mp[t] == -1:
                            mp[t] = qn
                            qn += 1
                        iters.append((v, t))
                        if not in_working[t]:
                            new_working[t] = True
                checked[v] = True
            working = [i for i in range(num_qubits) if new_working[i]]
            in_working = [False] * num_qubits
            for i in working:
                in_working[i] = True
            new_working = [False] * num_qubits
        real_iters.append([(mp[a], mp[b]) for a, b in iters])
        needed.append(qn)
    return real_iters, needed


def fmt(x):
    """ostream << double with default flags and precision 6."""
    return "%g" % x


def term_qasm(edges, num_qubits, p, betas_gammas):
    lines = [str(num_qubits)]
    lines += ["H %d" % i for i in range(num_qubits)]
    for i in range(p):
        gamma = betas_gammas[i + p]
        beta = betas_gammas[i]
        for a, b in edges:
            lines.append("CNOT %d %d" % (a, b))
            lines.append("Rz %s %d" % (fmt(-gamma), b))
            lines.append("CNOT %d %d" % (a, b))
        for j in range(num_qubits):
            lines.append("Rx %s %d" % (fmt(beta * 2.0), j))
    return "\n".join(lines) + "\n"


def term_measure(num_qubits):
    return "".join("Z " if i in (0, 1) else "T " for i in range(num_qubits))


def all_terms(dgf_text, p, betas_gammas):
    pairs, nq = read_dgf(dgf_text)
    iters, needed = light_cones(pairs, nq, p)
    return [(pairs[k], term_qasm(iters[k], needed[k], p, betas_gammas), term_measure(needed[k]))
            for k in range(len(pairs))]
