"""qtorch_gb300 — qTorch's tensor-network contraction engine on GB300 (sm_103a).

Python mirror of the C ABI (include/qtorch_gb300.h).  Every entry point runs on
the GPU through libqtorch_gb300.so; there is no CPU fallback: without the
library or without an sm_103 device, creating a context raises.

Names follow the reference API (src/Network.h, src/ContractionTools.h,
src/LineGraph.h) so that code written against qTorch reads the same:

    tools = ContractionTools("circuit.qasm", "measure.txt")
    tools.Contract(Stochastic, seed=7)
    value = tools.GetFinalVal()
"""
import ctypes
import os
import threading
import weakref

import numpy as np

from . import _capi

__all__ = [
    "QtError", "InvalidFile", "InvalidFileFormat", "ContractionFailure", "InvalidUserContractionSequence",
    "InvalidFunctionInput", "InvalidContractionMethod", "Refused", "DeadlineExpired", "OutOfMemory",
    "Context", "default_context", "contract_pair", "contract_pair_device", "Network", "ContractionTools",
    "LineGraph", "Plan", "Batch", "Server", "Stochastic", "FP64", "MIXED", "qaoa_term_text", "qaoa_num_edges",
    "random_regular_graph", "library_path",
]

FP64 = 0
MIXED = 1
Stochastic = 0
ORDER_STOCHASTIC, ORDER_LINEGRAPH, ORDER_SEQUENCE, ORDER_GREEDY, ORDER_AUTO = 0, 1, 2, 3, 4


class QtError(RuntimeError):
    status = -1

    def __init__(self, status, detail=""):
        self.status = status
        lib = _capi.load()
        msg = lib.qt_status_string(status).decode()
        super().__init__(f"{msg}{': ' + detail if detail else ''} (status {status})")


class InvalidFile(QtError):
    pass


class InvalidFileFormat(QtError):
    pass


class ContractionFailure(QtError):
    pass


class InvalidUserContractionSequence(QtError):
    pass


class InvalidFunctionInput(QtError):
    pass


class InvalidContractionMethod(QtError):
    pass


class Refused(QtError):
    pass


class OutOfMemory(QtError):
    pass


class DeadlineExpired(QtError):
    pass


_ERRORS = {2: InvalidFile, 3: InvalidFileFormat, 4: ContractionFailure, 5: InvalidUserContractionSequence,
           6: InvalidFunctionInput, 7: InvalidContractionMethod, 8: Refused, 9: OutOfMemory, 11: DeadlineExpired}


def library_path():
    return _capi.LIB_PATH


def _lib():
    return _capi.load()


def _check(status, ctx=None):
    if status != 0:
        detail = ""
        if ctx is not None and ctx.handle:
            buf = ctypes.create_string_buffer(512)
            _lib().qt_last_error(ctx.handle, buf, 512)
            detail = buf.value.decode(errors="replace")
        raise _ERRORS.get(status, QtError)(status, detail)


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class _Owned:
    """A native object tied to a context: the context frees it before it goes away."""

    _free_name = None
    _release_rank = 9   # lower ranks are freed first when the context closes

    def _register(self, ctx):
        if ctx is not None:
            ctx._deps.add(self)

    def _release(self):
        h = getattr(self, "handle", None)
        if h:
            self.handle = None
            getattr(_lib(), self._free_name)(h)

    def __del__(self):
        self._release()


class Context:
    """One device, one CUDA stream (``stream``: a cudaStream_t as int, or None)."""

    def __init__(self, device=0, stream=None):
        self.handle = None
        self._deps = weakref.WeakSet()
        h = ctypes.c_void_p()
        _check(_lib().qt_ctx_create(device, ctypes.c_void_p(stream) if stream else None, ctypes.byref(h)))
        self.handle = h.value
        self.device = device

    def close(self):
        if self.handle:
            # servers, batches, networks and plans on this context go first
            for dep in sorted(list(self._deps), key=lambda d: d._release_rank):
                dep._release()
            _lib().qt_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def synchronize(self):
        _check(_lib().qt_ctx_synchronize(self.handle), self)

    def set_memory_budget(self, nbytes):
        _check(_lib().qt_ctx_set_memory_budget(self.handle, int(nbytes)), self)

    def set_deadline(self, seconds):
        _check(_lib().qt_ctx_set_deadline(self.handle, float(seconds)), self)

    @property
    def kernel_launches(self):
        return int(_lib().qt_ctx_kernel_launches(self.handle))

    @property
    def tensor_core_steps(self):
        """contraction steps that ran on the tcgen05 tensor-core GEMM"""
        return int(_lib().qt_ctx_tensor_core_steps(self.handle))

    @property
    def stream_steps(self):
        """contraction steps that ran on the streaming kernel (small operand in shared memory)"""
        return int(_lib().qt_ctx_stream_steps(self.handle))

    def memory_stats(self):
        """(bytes in use, bytes cached, cudaMalloc calls so far) of the context's allocator"""
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(_lib().qt_ctx_memory_stats(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), self)
        return int(a.value), int(b.value), int(c.value)

    @property
    def last_error(self):
        buf = ctypes.create_string_buffer(512)
        _lib().qt_last_error(self.handle, buf, 512)
        return buf.value.decode(errors="replace")


_default = None
_default_lock = threading.Lock()


def default_context():
    global _default
    with _default_lock:
        if _default is None:
            _default = Context(0)
        return _default


def _index_maps(free_from_a, free_idx, sum_a, sum_b):
    ffa = np.ascontiguousarray(np.asarray(free_from_a, dtype=np.uint8))
    fi = np.ascontiguousarray(np.asarray(free_idx, dtype=np.int32))
    sa = np.ascontiguousarray(np.asarray(sum_a, dtype=np.int32))
    sb = np.ascontiguousarray(np.asarray(sum_b, dtype=np.int32))
    return ffa, fi, sa, sb


def _rank_of(n):
    r = 0
    while (1 << (2 * r)) < n:
        r += 1
    if (1 << (2 * r)) != n:
        raise ValueError(f"tensor of {n} elements is not 4^rank")
    return r


def contract_pair(a, b, free_from_a, free_idx, sum_a, sum_b, ctx=None):
    """ContractIndices (src/Network.h:876-971) of two host complex128 tensors on the GPU."""
    ctx = ctx or default_context()
    a = np.ascontiguousarray(a, dtype=np.complex128).reshape(-1)
    b = np.ascontiguousarray(b, dtype=np.complex128).reshape(-1)
    ffa, fi, sa, sb = _index_maps(free_from_a, free_idx, sum_a, sum_b)
    c = np.zeros(4 ** len(fi), dtype=np.complex128)
    _check(_lib().qt_contract_pair_host(
        ctx.handle, _dp(a.view(np.float64)), _rank_of(a.size), _dp(b.view(np.float64)), _rank_of(b.size), len(fi),
        ffa.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _ip(fi), len(sa), _ip(sa), _ip(sb),
        _dp(c.view(np.float64))), ctx)
    return c


def contract_pair_c64(a, b, free_from_a, free_idx, sum_a, sum_b, ctx=None):
    """The same contraction in complex64 through device tensors (qt_tensor_* and
    qt_contract_pair); GEMM-shaped steps run on the tcgen05 tensor cores."""
    ctx = ctx or default_context()
    lib = _lib()
    a = np.ascontiguousarray(a, dtype=np.complex64).reshape(-1)
    b = np.ascontiguousarray(b, dtype=np.complex64).reshape(-1)
    ffa, fi, sa, sb = _index_maps(free_from_a, free_idx, sum_a, sum_b)
    ta, tb, tc = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    try:
        _check(lib.qt_tensor_create(ctx.handle, _rank_of(a.size), 1, ctypes.byref(ta)), ctx)
        _check(lib.qt_tensor_create(ctx.handle, _rank_of(b.size), 1, ctypes.byref(tb)), ctx)
        _check(lib.qt_tensor_upload(ctx.handle, ta, a.ctypes.data_as(ctypes.c_void_p), a.nbytes), ctx)
        _check(lib.qt_tensor_upload(ctx.handle, tb, b.ctypes.data_as(ctypes.c_void_p), b.nbytes), ctx)
        _check(lib.qt_contract_pair(ctx.handle, ta, tb, len(fi), ffa.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                    _ip(fi), len(sa), _ip(sa), _ip(sb), ctypes.byref(tc)), ctx)
        c = np.zeros(4 ** len(fi), dtype=np.complex64)
        _check(lib.qt_tensor_download(ctx.handle, tc, c.ctypes.data_as(ctypes.c_void_p), c.nbytes), ctx)
        return c
    finally:
        for t in (ta, tb, tc):
            if t.value:
                lib.qt_tensor_free(ctx.handle, t)


def permute(x, perm, ctx=None):
    """Index permutation of a host tensor on the GPU (qt_tensor_permute): digit
    i of the result's flat index is digit perm[i] of x's.  complex64 stays
    complex64; anything else runs as complex128."""
    ctx = ctx or default_context()
    lib = _lib()
    c64 = np.asarray(x).dtype == np.complex64
    x = np.ascontiguousarray(x, dtype=np.complex64 if c64 else np.complex128).reshape(-1)
    pa = np.ascontiguousarray(np.asarray(perm, dtype=np.int32))
    tx, ty = ctypes.c_void_p(), ctypes.c_void_p()
    try:
        _check(lib.qt_tensor_create(ctx.handle, _rank_of(x.size), 1 if c64 else 0, ctypes.byref(tx)), ctx)
        _check(lib.qt_tensor_upload(ctx.handle, tx, x.ctypes.data_as(ctypes.c_void_p), x.nbytes), ctx)
        _check(lib.qt_tensor_permute(ctx.handle, tx, _ip(pa) if pa.size else None, ctypes.byref(ty)), ctx)
        y = np.empty_like(x)
        _check(lib.qt_tensor_download(ctx.handle, ty, y.ctypes.data_as(ctypes.c_void_p), y.nbytes), ctx)
        return y
    finally:
        for t in (tx, ty):
            if t.value:
                lib.qt_tensor_free(ctx.handle, t)


def contract_pair_device(a_ptr, rank_a, b_ptr, rank_b, free_from_a, free_idx, sum_a, sum_b, c_ptr, ctx=None):
    """ContractIndices on caller-owned device buffers (complex128), asynchronous on ctx's stream."""
    ctx = ctx or default_context()
    ffa, fi, sa, sb = _index_maps(free_from_a, free_idx, sum_a, sum_b)
    _check(_lib().qt_contract_pair_device(
        ctx.handle, ctypes.c_void_p(a_ptr), rank_a, ctypes.c_void_p(b_ptr), rank_b, len(fi),
        ffa.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _ip(fi), len(sa), _ip(sa), _ip(sb),
        ctypes.c_void_p(c_ptr)), ctx)


class Network(_Owned):
    """Network (src/Network.h:54-140): parse, ContractNodes on the GPU, final value."""

    _free_name = "qt_network_free"
    _release_rank = 2

    def __init__(self, qasm_text, measure_text="", gate_dir=None, ctx=None, symbolic=False):
        self.ctx = None if symbolic else (ctx or default_context())
        h = ctypes.c_void_p()
        _check(_lib().qt_network_create(self.ctx.handle if self.ctx else None, qasm_text.encode(),
                                        (measure_text or "").encode(), gate_dir.encode() if gate_dir else None,
                                        ctypes.byref(h)), self.ctx)
        self.handle = h.value
        self._register(self.ctx)

    @classmethod
    def from_files(cls, qasm_path, measure_path, ctx=None):
        with open(qasm_path) as f:
            q = f.read()
        try:
            with open(measure_path) as f:
                m = f.read()
        except OSError:
            m = ""   # every qubit traced out, as Network.h:286-288
        return cls(q, m, gate_dir=None, ctx=ctx)

    def reset(self):
        _check(_lib().qt_network_reset(self.handle), self.ctx)

    @property
    def num_qubits(self):
        return _lib().qt_network_num_qubits(self.handle)

    @property
    def num_nodes(self):
        return _lib().qt_network_num_nodes(self.handle)

    @property
    def num_uncontracted(self):
        return _lib().qt_network_num_uncontracted(self.handle)

    def node_rank(self, i):
        return _lib().qt_network_node_rank(self.handle, i)

    @property
    def is_done(self):
        return bool(_lib().qt_network_is_done(self.handle))

    def contract_nodes(self, a, b, threshold):
        out = ctypes.c_int(-1)
        _check(_lib().qt_network_contract_nodes(self.handle, a, b, threshold, ctypes.byref(out)), self.ctx)
        return None if out.value < 0 else out.value

    def contract_sequence(self, pairs):
        arr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1))
        _check(_lib().qt_network_contract_sequence(self.handle, _ip(arr), arr.size // 2), self.ctx)

    def contract_user_sequence(self, text):
        _check(_lib().qt_network_contract_user_sequence(self.handle, text.encode()), self.ctx)

    def contract_stochastic(self, seed):
        _check(_lib().qt_network_contract_stochastic(self.handle, int(seed)), self.ctx)

    def contract_linegraph(self):
        _check(_lib().qt_network_contract_linegraph(self.handle), self.ctx)

    def contract_wire_order(self, order_1based):
        arr = np.ascontiguousarray(np.asarray(order_1based, dtype=np.int32))
        _check(_lib().qt_network_contract_wire_order(self.handle, _ip(arr), arr.size), self.ctx)

    def linegraph_order(self):
        n = _lib().qt_network_linegraph_order(self.handle, None, 0)
        arr = np.zeros(max(n, 1), dtype=np.int32)
        _lib().qt_network_linegraph_order(self.handle, _ip(arr), n)
        return [int(x) for x in arr[:n]]

    def reduce(self):
        _check(_lib().qt_network_reduce(self.handle), self.ctx)

    @property
    def final_value(self):
        v = np.zeros(2)
        _check(_lib().qt_network_final_value(self.handle, _dp(v)), self.ctx)
        return complex(v[0], v[1])

    @property
    def flops(self):
        return int(_lib().qt_network_flops(self.handle))

    def created_from(self):
        n = _lib().qt_network_created_from(self.handle, None, 0)
        arr = np.zeros(2 * max(n, 1), dtype=np.int32)
        _lib().qt_network_created_from(self.handle, _ip(arr), n)
        return [(int(arr[2 * i]), int(arr[2 * i + 1])) for i in range(n)]

    def node_values(self, i):
        n = _lib().qt_network_node_values(self.handle, i, None, 0)
        if n < 0:
            return None
        out = np.zeros(n, dtype=np.complex128)
        _lib().qt_network_node_values(self.handle, i, _dp(out.view(np.float64)), n)
        return out


class ContractionTools:
    """ContractionTools (src/ContractionTools.h:52-123) over a GPU-backed Network."""

    def __init__(self, qasm_or_network, measure_path=None, ctx=None):
        if isinstance(qasm_or_network, Network):
            self._net = qasm_or_network
            self._paths = None
        else:
            self._net = None
            self._paths = (qasm_or_network, measure_path)
        self._ctx = ctx
        self._final = 0j

    def _acquire(self):
        if self._net is None:
            self._net = Network.from_files(*self._paths, ctx=self._ctx)
        return self._net

    def Contract(self, kind=Stochastic, seed=None):
        if kind != Stochastic:
            raise InvalidContractionMethod(7)
        net = self._acquire()
        net.contract_stochastic(np.random.SeedSequence().entropy % (1 << 63) if seed is None else seed)
        self._final = net.final_value
        return net

    def ContractGivenSequence(self, sequence):
        net = self._acquire()
        net.contract_sequence(sequence)
        self._final = net.final_value
        return net

    def ContractUserDefinedSequenceOfWires(self, path):
        with open(path) as f:
            text = f.read()
        net = self._acquire()
        net.contract_user_sequence(text)
        self._final = net.final_value
        return net

    def GetFinalVal(self):
        return self._final


class LineGraph:
    """LineGraph (src/LineGraph.h): min-fill elimination order of the line graph, then LGContract."""

    def __init__(self, network):
        self._net = network

    def ordering(self):
        return self._net.linegraph_order()

    def LGContract(self, order_1based=None):
        if order_1based is None:
            self._net.contract_linegraph()
        else:
            self._net.contract_wire_order(order_1based)
        return True


_ORDER_NAMES = {"stochastic": ORDER_STOCHASTIC, "linegraph": ORDER_LINEGRAPH, "sequence": ORDER_SEQUENCE,
                "greedy": ORDER_GREEDY, "auto": ORDER_AUTO}


class Plan(_Owned):
    """An ordering lowered once; executed for many leaf bindings (see qt_plan_build)."""

    _free_name = "qt_plan_free"
    _release_rank = 3

    def __init__(self, qasm_text, measure_text="", ordering="linegraph", seed=0, sequence=None, gate_dir=None,
                 ctx=None, symbolic=False, tries=100, max_macs=0):
        """ordering: "linegraph", "stochastic" (seeded), "sequence" (recorded
        node-id pairs), "greedy" (size-greedy merges, best of 4096 seeded tries:
        for networks too large for min-fill), "auto" (greedy, or min-fill where
        the line graph is small and its walk is better) or "search" -- the preProcess-style search
        (qt_plan_build_search): `tries` seeded stochastic orderings from `seed`,
        the one with the smallest largest intermediate, then fewest MACs, kept
        (its seed in `chosen_seed`)."""
        # symbolic plans need no device: they can be inspected but not executed
        self.ctx = None if symbolic else (ctx or default_context())
        self.chosen_seed = None
        h = ctypes.c_void_p()
        if ordering == "search":
            cs = ctypes.c_uint64()
            _check(_lib().qt_plan_build_search(self.ctx.handle if self.ctx else None, qasm_text.encode(),
                                               (measure_text or "").encode(), gate_dir.encode() if gate_dir else None,
                                               int(seed), int(tries), int(max_macs), ctypes.byref(h),
                                               ctypes.byref(cs)), self.ctx)
            self.chosen_seed = int(cs.value)
        else:
            seq = np.ascontiguousarray(np.asarray(sequence if sequence is not None else [], dtype=np.int32).reshape(-1))
            _check(_lib().qt_plan_build(self.ctx.handle if self.ctx else None, qasm_text.encode(),
                                        (measure_text or "").encode(),
                                        gate_dir.encode() if gate_dir else None, _ORDER_NAMES[ordering], int(seed),
                                        _ip(seq) if seq.size else None, seq.size // 2, ctypes.byref(h)), self.ctx)
        self.handle = h.value
        self._register(self.ctx)

    @property
    def num_steps(self):
        return _lib().qt_plan_num_steps(self.handle)

    @property
    def item_descriptors(self):
        """work items of the mixed form with a host-prepared descriptor"""
        return int(_lib().qt_plan_item_descriptors(self.handle))

    @property
    def num_leaves(self):
        return _lib().qt_plan_num_leaves(self.handle)

    @property
    def peak_rank(self):
        return _lib().qt_plan_peak_rank(self.handle)

    def workspace_bytes(self, precision=FP64):
        return int(_lib().qt_plan_workspace_bytes(self.handle, precision))

    @property
    def flops(self):
        return int(_lib().qt_plan_flops(self.handle))

    def algorithmic_bytes(self, precision=FP64):
        return int(_lib().qt_plan_algorithmic_bytes(self.handle, precision))

    def sequence(self):
        n = _lib().qt_plan_sequence(self.handle, None, 0)
        arr = np.zeros(2 * max(n, 1), dtype=np.int32)
        _lib().qt_plan_sequence(self.handle, _ip(arr), n)
        return [(int(arr[2 * i]), int(arr[2 * i + 1])) for i in range(n)]

    def leaf_values(self):
        n = int(_lib().qt_plan_leaf_elems(self.handle))
        out = np.zeros(n, dtype=np.complex128)
        _check(_lib().qt_plan_leaf_values(self.handle, _dp(out.view(np.float64)), n), self.ctx)
        return out

    def execute(self, precision=FP64):
        v = np.zeros(2)
        _check(_lib().qt_plan_execute(self.ctx.handle, self.handle, precision, _dp(v)), self.ctx)
        return complex(v[0], v[1])

    def slice(self, max_workspace_bytes, precision=FP64, max_cuts=8):
        """Index slicing under a workspace budget (qt_plan_slice)."""
        return SlicedPlan(self, max_workspace_bytes, precision, max_cuts)

    @property
    def num_rotations(self):
        return _lib().qt_plan_num_rotations(self.handle)

    def rotation_angles(self):
        n = self.num_rotations
        out = np.zeros(max(n, 1))
        _check(_lib().qt_plan_rotation_angles(self.handle, _dp(out), n), self.ctx)
        return out[:n].copy()

    STEP_INFO_FIELDS = ("level", "rank_a", "rank_b", "rank_c", "summed", "group", "flags", "table")

    def step_info(self, precision=FP64):
        """The interpreter schedule: one row per step in execution order with the
        columns of STEP_INFO_FIELDS."""
        n = self.num_steps
        out = np.zeros((max(n, 1), len(self.STEP_INFO_FIELDS)), dtype=np.int32)
        got = _lib().qt_plan_step_info(self.handle, precision,
                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), n)
        if got < 0:
            raise InvalidFunctionInput("qt_plan_step_info")
        return out[:n].copy()


class SlicedPlan(_Owned):
    """A plan split over the values of a few cut wires (qt_plan_slice)."""

    _free_name = "qt_sliced_free"
    _release_rank = 1

    def __init__(self, plan, max_workspace_bytes, precision=FP64, max_cuts=8):
        self.ctx = plan.ctx
        self.plan = plan
        h = ctypes.c_void_p()
        _check(_lib().qt_plan_slice(self.ctx.handle if self.ctx else None, plan.handle, precision,
                                    int(max_workspace_bytes), int(max_cuts), ctypes.byref(h)), self.ctx)
        self.handle = h.value
        self._register(self.ctx)

    @property
    def num_cuts(self):
        return _lib().qt_sliced_num_cuts(self.handle)

    @property
    def num_slices(self):
        return 4 ** self.num_cuts

    def workspace_bytes(self, precision=FP64):
        """workspace of one slice"""
        return int(_lib().qt_plan_workspace_bytes(_lib().qt_sliced_plan(self.handle), precision))

    @property
    def slice_flops(self):
        return int(_lib().qt_plan_flops(_lib().qt_sliced_plan(self.handle)))

    def execute(self, precision=FP64, leaves=None):
        """Sum over the slices; `leaves`: other values of the uncut plan's leaves
        (complex128, its leaf order), every slice then step by step."""
        v = np.zeros(2)
        if leaves is None:
            _check(_lib().qt_sliced_execute(self.handle, precision, _dp(v)), self.ctx)
        else:
            lv = np.ascontiguousarray(leaves, dtype=np.complex128)
            _check(_lib().qt_sliced_execute_leaves(self.ctx.handle, self.handle, precision, _dp(lv.view(np.float64)),
                                                   _dp(v)), self.ctx)
        return complex(v[0], v[1])


class Batch(_Owned):
    """Many plan instances in one persistent grouped launch."""

    _free_name = "qt_batch_free"
    _release_rank = 1

    def __init__(self, ctx=None):
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        _check(_lib().qt_batch_create(self.ctx.handle, ctypes.byref(h)), self.ctx)
        self.handle = h.value
        self._plans = []
        self._eval = None   # evaluate(): angle and value buffers with their addresses
        self._eval_lock = threading.Lock()
        self._register(self.ctx)

    def add(self, plan, leaves=None):
        idx = ctypes.c_int(-1)
        if leaves is not None:
            leaves = np.ascontiguousarray(leaves, dtype=np.complex128)
        _check(_lib().qt_batch_add(self.handle, plan.handle,
                                   _dp(leaves.view(np.float64)) if leaves is not None else None,
                                   ctypes.byref(idx)), self.ctx)
        self._plans.append(plan)
        return idx.value

    def __len__(self):
        return _lib().qt_batch_size(self.handle)

    def execute(self, precision=FP64):
        out = np.zeros(2 * len(self))
        _check(_lib().qt_batch_execute(self.handle, precision, _dp(out)), self.ctx)
        return out.view(np.complex128).copy()

    def prepare(self, precision=FP64):
        _check(_lib().qt_batch_prepare(self.handle, precision), self.ctx)

    def run(self):
        _check(_lib().qt_batch_run(self.handle), self.ctx)

    def fetch(self):
        out = np.zeros(2 * len(self))
        _check(_lib().qt_batch_fetch(self.handle, _dp(out)), self.ctx)
        return out.view(np.complex128).copy()

    def set_leaves(self, index, leaves):
        leaves = np.ascontiguousarray(leaves, dtype=np.complex128)
        _check(_lib().qt_batch_set_leaves(self.handle, index, _dp(leaves.view(np.float64))), self.ctx)

    def set_rotations(self, angles):
        a = np.ascontiguousarray(np.asarray(angles, dtype=np.float64))
        _check(_lib().qt_batch_set_rotations(self.handle, _dp(a), a.size), self.ctx)

    def evaluate(self, angles=None):
        """Values of every instance at new rotation angles in one call (gate
        tensors built on the device; the batch must be prepared for MIXED when
        angles are given)."""
        if angles is None:
            out = np.empty(len(self._plans), dtype=np.complex128)
            st = _lib().qt_batch_evaluate(self.handle, None, 0, out.ctypes.data)
            if st:
                _check(st, self.ctx)
            return out
        # The call is short (~10 us through the resident engine), so the
        # wrapper keeps one angle and one value buffer per batch and their
        # addresses (reading an array's .ctypes address costs about a
        # microsecond); the lock keeps concurrent callers off each other's buffers.
        with self._eval_lock:
            e = self._eval
            n = np.size(angles)
            if e is None or e[0].size != n or e[2].size != len(self._plans):
                ang = np.empty(n, dtype=np.float64)
                out = np.empty(len(self._plans), dtype=np.complex128)
                e = self._eval = (ang, ang.ctypes.data, out, out.ctypes.data, _lib().qt_batch_evaluate)
            e[0][:] = np.ravel(angles)
            st = e[4](self.handle, e[1], n, e[3])
            if st:
                _check(st, self.ctx)
            return e[2].copy()

    def set_rotations_device(self, angles):
        """New rotation angles whose gate tensors are built on the device at the
        next run (batches prepared for MIXED); only the angles are copied."""
        a = np.ascontiguousarray(np.asarray(angles, dtype=np.float64))
        _check(_lib().qt_batch_set_rotations_device(self.handle, _dp(a), a.size), self.ctx)

    def upload(self):
        _check(_lib().qt_batch_upload(self.handle), self.ctx)

    def use_graph(self, enable=True):
        _check(_lib().qt_batch_use_graph(self.handle, 1 if enable else 0), self.ctx)

    def use_resident(self, idle_seconds=0.5):
        """Keep one CTA per instance on the GPU between evaluate() calls
        (qt_batch_use_resident); 0 stops it."""
        _check(_lib().qt_batch_use_resident(self.handle, float(idle_seconds)), self.ctx)

    @property
    def resident_starts(self):
        """launches of the resident engine so far"""
        return int(_lib().qt_batch_resident_starts(self.handle))

    @property
    def h2d_bytes(self):
        return int(_lib().qt_batch_h2d_bytes(self.handle))

    @property
    def d2h_bytes(self):
        return int(_lib().qt_batch_d2h_bytes(self.handle))

    @property
    def launches_per_run(self):
        return int(_lib().qt_batch_launches_per_run(self.handle))

    @property
    def launch_policy(self):
        """dict of qt_launch_policy (negative caps: defaults)"""
        pol = _capi.LaunchPolicy()
        _check(_lib().qt_batch_get_launch_policy(self.handle, ctypes.byref(pol)), self.ctx)
        return {k: getattr(pol, k) for k, _ in pol._fields_}

    def set_launch_policy(self, ws_smem_cap=-1, stage_cap=-1, ctas_per_sm=0, static_schedule=0, kernel_ctas=0):
        pol = _capi.LaunchPolicy(ws_smem_cap, stage_cap, ctas_per_sm, static_schedule, kernel_ctas)
        _check(_lib().qt_batch_set_launch_policy(self.handle, ctypes.byref(pol)), self.ctx)

    def launch_info(self):
        """dict of qt_launch_info for the prepared batch"""
        info = _capi.LaunchInfo()
        _check(_lib().qt_batch_launch_info(self.handle, ctypes.byref(info)), self.ctx)
        return {k: getattr(info, k) for k, _ in info._fields_}

    def autotune(self, reps=3):
        """Time candidate launch policies on the prepared batch and keep the
        fastest; returns (policy dict, microseconds per grouped launch)."""
        pol = _capi.LaunchPolicy()
        us = ctypes.c_double()
        _check(_lib().qt_batch_autotune(self.handle, reps, ctypes.byref(pol), ctypes.byref(us)), self.ctx)
        return {k: getattr(pol, k) for k, _ in pol._fields_}, us.value


class Server(_Owned):
    """Continuous-batching request loop (qt_server_*)."""

    _free_name = "qt_server_free"
    _release_rank = 0

    def __init__(self, max_inflight=64, precision=FP64, ctx=None, max_macs=0):
        """max_macs > 0: requests of more complex MACs (over all slices) are
        refused at submission (submit raises Refused)."""
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        _check(_lib().qt_server_create(self.ctx.handle, max_inflight, precision, ctypes.byref(h)), self.ctx)
        self.handle = h.value
        self._keep = []
        self._register(self.ctx)
        if max_macs:
            self.set_max_macs(max_macs)

    def set_max_macs(self, max_macs):
        _check(_lib().qt_server_set_max_macs(self.handle, int(max_macs)), self.ctx)

    def close(self):
        self._release()

    def submit(self, plan, leaves=None):
        t = ctypes.c_int64(-1)
        if leaves is not None:
            leaves = np.ascontiguousarray(leaves, dtype=np.complex128)
        self._keep.append(plan)
        _check(_lib().qt_server_submit(self.handle, plan.handle,
                                       _dp(leaves.view(np.float64)) if leaves is not None else None,
                                       ctypes.byref(t)), self.ctx)
        return t.value

    def poll(self, ticket):
        v = np.zeros(2)
        lat = ctypes.c_double(0)
        st = _lib().qt_server_poll(self.handle, ticket, _dp(v), ctypes.byref(lat))
        if st < 0:
            raise _ERRORS.get(-st, QtError)(-st)
        return (complex(v[0], v[1]), lat.value) if st == 1 else None

    def poll_detail(self, ticket):
        """(value, latency, seconds queued before admission, lane) or None while pending"""
        v = np.zeros(2)
        lat, q, lane = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_int(-1)
        st = _lib().qt_server_poll_detail(self.handle, ticket, _dp(v), ctypes.byref(lat), ctypes.byref(q),
                                          ctypes.byref(lane))
        if st < 0:
            raise _ERRORS.get(-st, QtError)(-st)
        return (complex(v[0], v[1]), lat.value, q.value, lane.value) if st == 1 else None

    def drain(self):
        _check(_lib().qt_server_drain(self.handle), self.ctx)

    def stats(self):
        p50, p99 = ctypes.c_double(0), ctypes.c_double(0)
        done, launches = ctypes.c_int64(0), ctypes.c_int64(0)
        _check(_lib().qt_server_stats(self.handle, ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(done),
                                      ctypes.byref(launches)), self.ctx)
        waves, reqs, secs = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_double(0)
        _check(_lib().qt_server_wave_stats(self.handle, ctypes.byref(waves), ctypes.byref(reqs), ctypes.byref(secs)),
               self.ctx)
        return {"p50_s": p50.value, "p99_s": p99.value, "completed": done.value, "launches": launches.value,
                "waves": waves.value, "wave_requests": reqs.value, "lane_seconds": secs.value,
                "refused": int(_lib().qt_server_refused(self.handle)),
                "oom_retries": int(_lib().qt_server_oom_retries(self.handle))}


def qaoa_num_edges(dgf_text):
    return _lib().qt_qaoa_num_edges(dgf_text.encode())


def qaoa_term_text(dgf_text, p, betas_gammas, edge):
    """(qasm, measure) of one MaxCut light-cone term, as src/maxcut.cpp:166-190 writes it."""
    bg = np.ascontiguousarray(np.asarray(betas_gammas, dtype=np.float64))
    n = _lib().qt_qaoa_term_text(dgf_text.encode(), p, _dp(bg), edge, None, 0, None, 0)
    if n < 0:
        raise ValueError("bad graph, p or edge")
    q = ctypes.create_string_buffer(int(n))
    m = ctypes.create_string_buffer(4096)
    _lib().qt_qaoa_term_text(dgf_text.encode(), p, _dp(bg), edge, q, int(n), m, 4096)
    return q.value.decode(), m.value.decode()


def qaoa_circuit_text(dgf_text, p, betas_gammas):
    """The whole MaxCut QAOA circuit of a graph (src/maxcut.cpp:52-56)."""
    bg = np.ascontiguousarray(np.asarray(betas_gammas, dtype=np.float64))
    n = _lib().qt_qaoa_circuit_text(dgf_text.encode(), p, _dp(bg), None, 0)
    if n < 0:
        raise ValueError("bad graph or p")
    q = ctypes.create_string_buffer(int(n))
    _lib().qt_qaoa_circuit_text(dgf_text.encode(), p, _dp(bg), q, int(n))
    return q.value.decode()


def random_regular_graph(num_nodes, degree, seed):
    n = _lib().qt_random_regular_graph(num_nodes, degree, int(seed), None, 0)
    if n < 0:
        raise ValueError("no regular graph for these parameters")
    buf = ctypes.create_string_buffer(int(n))
    _lib().qt_random_regular_graph(num_nodes, degree, int(seed), buf, int(n))
    return buf.value.decode()


def run_inp(path, ctx=None, symbolic=False):
    """Run an .inp script (src/main.cpp flow): returns (value, flop counter)."""
    c = None if symbolic else (ctx or default_context())
    v = np.zeros(2)
    fl = ctypes.c_int64(0)
    _check(_lib().qt_run_inp(c.handle if c else None, path.encode(), _dp(v), ctypes.byref(fl)), c)
    return complex(v[0], v[1]), fl.value


from .maxcut import MaxCutQAOA, maxcut_final_string  # noqa: E402,F401
