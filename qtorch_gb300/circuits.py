"""QASM text of the circuit families the serving workload mixes (in the
reference's QASM dialect, src/Network.h:326-707)."""
import math

import numpy as np


def qft_text(n, seed):
    """QFT on n qubits from a random computational-basis input (X on a seeded
    subset), laid out like the reference's Samples/qft*.qasm: H and a ladder of
    CRk per qubit, then the qubit-reversal swaps (three CNOTs each)."""
    rng = np.random.default_rng(seed)
    lines = [str(n)]
    for q in range(n):
        if rng.integers(2):
            lines.append(f"X {q}")
    for i in range(n):
        lines.append(f"H {i}")
        for j in range(i + 1, n):
            lines.append(f"CRk {j} {i}")
    for i in range(n // 2):
        a, b = i, n - 1 - i
        lines += [f"CNOT {a} {b}", f"CNOT {b} {a}", f"CNOT {a} {b}"]
    return "\n".join(lines) + "\n"


def qft_measure_text(n):
    """<X> on the last qubit, traces elsewhere.  The QFT of a basis state |x> is
    a product state: <Z> is 0 on every qubit and qubit 0 (after the reversal
    swaps) carries the phase pi*x, so <X_0> = +-1; the last qubit carries
    2 pi x / 2^n, a generic value."""
    return " ".join(["T"] * (n - 1) + ["X"])


def config1_circuit_text(seed, n=6, depth=10, cz_pairs=2):
    """Each layer: Rx(theta), theta ~ U[0, 2 pi), on every qubit, then CZ on
    `cz_pairs` random disjoint qubit pairs (seeded)."""
    rng = np.random.default_rng(seed)
    lines = [str(n)]
    for _ in range(depth):
        for q in range(n):
            lines.append(f"Rx {rng.uniform(0, 2 * math.pi):.6f} {q}")
        perm = rng.permutation(n)
        for j in range(cz_pairs):
            lines.append(f"CZ {perm[2 * j]} {perm[2 * j + 1]}")
    return "\n".join(lines) + "\n"


def random_circuit_text(n, depth, seed):
    """Layers of seeded Rx/Ry/Rz on every qubit, then CZ on n/4 disjoint random pairs."""
    rng = np.random.default_rng(seed)
    lines = [str(n)]
    for _ in range(depth):
        for q in range(n):
            lines.append(f"{rng.choice(['Rx', 'Ry', 'Rz'])} {rng.uniform(0, 2 * math.pi):.4f} {q}")
        perm = rng.permutation(n)
        for j in range(0, n // 4 * 2, 2):
            lines.append(f"CZ {perm[j]} {perm[j + 1]}")
    return "\n".join(lines) + "\n"
