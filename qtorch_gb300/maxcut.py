"""MaxCut QAOA driver on the batched engine: the objective and angle search of
maxcutGetOptimalAngles (src/maxcut.cpp:144-225) and the final-cut decoding of
maxcutGetFinalString (src/maxcut.cpp:29-140).

The reference re-writes and re-parses one QASM file per edge term for every
objective call and contracts it with a fresh stochastic ordering.  Here every
term is lowered once (line-graph ordering by default) and one objective call is
one batched evaluation of all terms at the new angles: only the rotation angles
travel, the gate tensors are built on the device, and with ``resident=True`` the
terms' CTAs stay on the GPU between calls (``qt_batch_use_resident``).

The optimiser is COBYLA, as in the reference (nlopt's LN_COBYLA, maximising
F_p from betas = 0.392699, gammas = 0.785399).  nlopt is not part of this
build; SciPy's COBYLA implementation of the same method (Powell 1994) is used
when SciPy is importable.
"""
import ctypes

import numpy as np

# starting point of maxcutGetOptimalAngles (src/maxcut.cpp:154-156)
START_BETA = 0.392699
START_GAMMA = 0.785399


def _term_shape(qasm_text, p):
    """(light-cone edges per layer, qubits) of a term: its rotations come as
    [Rz(-gamma_i) x edges, Rx(2 beta_i) x qubits] for i = 1..p
    (applyU_CsThenU_Bs, src/maxcut.h:205-233)."""
    n = int(qasm_text.split("\n", 1)[0])
    n_rz = sum(1 for line in qasm_text.split("\n") if line.startswith("Rz "))
    return n_rz // p, n


def rotation_angles(shapes, betas_gammas, p):
    """Rotation angles of every term at one point, in leaf order, as the
    reference's text carries them (6 significant digits) and its parser reads
    them."""
    betas, gammas = betas_gammas[:p], betas_gammas[p:]
    out = []
    for e, n in shapes:
        for i in range(p):
            out += [float("%g" % -gammas[i])] * e + [float("%g" % (betas[i] * 2.0))] * n
    return np.array(out, dtype=np.float64)


class MaxCutQAOA:
    """F_p(betas, gammas) = sum over edges of 0.5 (1 - <Z_a Z_b>) for a .dgf
    graph, each edge's light-cone term a plan of one batch."""

    def __init__(self, dgf_text, p, precision=None, ordering="linegraph", ctx=None, resident=True, autotune=True):
        from . import MIXED, Batch, Plan, default_context, qaoa_num_edges, qaoa_term_text
        self.dgf = dgf_text
        self.p = p
        self.precision = MIXED if precision is None else precision
        self.ctx = ctx or default_context()
        self.n_edges = qaoa_num_edges(dgf_text)
        start = [START_BETA] * p + [START_GAMMA] * p
        self.plans, self.shapes = [], []
        self.batch = Batch(self.ctx)
        for e in range(self.n_edges):
            qasm, meas = qaoa_term_text(dgf_text, p, start, e)
            pl = Plan(qasm, meas, ordering=ordering, seed=e + 1, ctx=self.ctx)
            self.plans.append(pl)
            self.shapes.append(_term_shape(qasm, p))
            self.batch.add(pl)
        self.batch.prepare(self.precision)
        self.batch.use_graph(True)
        if autotune:
            self.batch.autotune()
        self.device_rotations = self.precision == MIXED
        if resident and self.device_rotations:
            self.batch.use_resident(0.5)
        self.evaluations = 0

    def term_values(self, betas_gammas):
        """<Z_a Z_b> of every edge at the point."""
        a = rotation_angles(self.shapes, list(betas_gammas), self.p)
        self.evaluations += 1
        if self.device_rotations:
            return self.batch.evaluate(a)
        self.batch.set_rotations(a)   # FP64: the reference's gate tables, built on the host
        return self.batch.execute(self.precision)

    def objective(self, betas_gammas):
        """F_p at the point (src/maxcut.cpp:188: f_pVal += 0.5 (1 - Re <ZZ>))."""
        return float(np.sum(0.5 * (1.0 - self.term_values(betas_gammas).real)))

    def optimize(self, x0=None, rhobeg=0.5, tol=1e-6, maxiter=200):
        """Maximise F_p with COBYLA from the reference's starting point.
        Returns (betas_gammas, F_p)."""
        try:
            from scipy.optimize import minimize
        except ImportError as e:   # pragma: no cover - SciPy is on both machines
            raise RuntimeError("the COBYLA search needs SciPy") from e
        x0 = np.array([START_BETA] * self.p + [START_GAMMA] * self.p if x0 is None else x0, dtype=np.float64)
        res = minimize(lambda x: -self.objective(x), x0, method="COBYLA",
                       options={"rhobeg": rhobeg, "tol": tol, "maxiter": maxiter})
        return np.asarray(res.x), -float(res.fun)

    def final_string(self, betas_gammas, precision=None, ordering="linegraph", seed=0):
        """Decode a cut from the whole circuit at the point (see maxcut_final_string)."""
        from . import FP64
        return maxcut_final_string(self.dgf, self.p, betas_gammas, FP64 if precision is None else precision,
                                   ordering=ordering, seed=seed, ctx=self.ctx)

    def close(self):
        self.batch.use_resident(0)


def maxcut_final_string(dgf_text, p, betas_gammas, precision, ordering="linegraph", seed=0, ctx=None,
                        marginals=False):
    """qt_maxcut_final_string: (bits, cut edges, probability of the string),
    plus the per-query values P(bits before i, bit i = 0) with marginals=True."""
    from . import _ORDER_NAMES, _check, _lib, default_context, qaoa_circuit_text
    ctx = ctx or default_context()
    n_max = int(qaoa_circuit_text(dgf_text, p, betas_gammas).split("\n", 1)[0])   # vertices
    bg = np.ascontiguousarray(np.asarray(betas_gammas, dtype=np.float64))
    bits = np.zeros(n_max, dtype=np.int32)
    n_bits, cut = ctypes.c_int(), ctypes.c_int()
    prob = ctypes.c_double()
    marg = np.zeros(n_max)
    _check(_lib().qt_maxcut_final_string(
        ctx.handle, dgf_text.encode(), p, bg.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), precision,
        _ORDER_NAMES[ordering], seed, bits.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), n_max,
        ctypes.byref(n_bits), ctypes.byref(cut), ctypes.byref(prob),
        marg.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), ctx)
    out = [int(b) for b in bits[:n_bits.value]], cut.value, prob.value
    return out + (marg[:n_bits.value].copy(),) if marginals else out

