"""ctypes binding of oracle/qt_oracle.c — TEST INFRASTRUCTURE ONLY (see oracle/__init__.py)."""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libqt_oracle.so")
_lib = None

QTO_OK = 0
QTO_INVALID_FILE = 1
QTO_INVALID_FILE_FORMAT = 2
QTO_CONTRACTION_FAILURE = 3
QTO_INVALID_FUNCTION_INPUT = 4


class OracleError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"oracle error {code} {msg}")
        self.code = code


def build():
    """Compile qt_oracle.c with the committed Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        d, i, c = ctypes.c_double, ctypes.c_int, ctypes.c_char_p
        L.qto_contract_indices.argtypes = [i, P(d), i, P(d), i, P(i), P(i), i, P(i), P(i), P(d)]
        L.qto_contract_indices.restype = None
        L.qto_gate_tensor.argtypes = [c, d, P(d)]
        L.qto_gate_tensor.restype = i
        L.qto_arbitrary_gate.argtypes = [c, i, P(d)]
        L.qto_arbitrary_gate.restype = i
        L.qto_net_parse.argtypes = [c, c, c, P(i)]
        L.qto_net_parse.restype = ctypes.c_void_p
        L.qto_net_free.argtypes = [ctypes.c_void_p]
        for name in ("qto_net_num_qubits", "qto_net_num_nodes", "qto_net_done"):
            getattr(L, name).argtypes = [ctypes.c_void_p]
            getattr(L, name).restype = i
        L.qto_net_node_rank.argtypes = [ctypes.c_void_p, i]
        L.qto_net_node_rank.restype = i
        L.qto_net_node_values.argtypes = [ctypes.c_void_p, i, P(d), ctypes.c_int64]
        L.qto_net_node_values.restype = i
        L.qto_net_contract.argtypes = [ctypes.c_void_p, i, i, i]
        L.qto_net_contract.restype = i
        L.qto_net_replay.argtypes = [ctypes.c_void_p, P(i), i]
        L.qto_net_replay.restype = i
        L.qto_net_lg_contract.argtypes = [ctypes.c_void_p, P(i), i]
        L.qto_net_lg_contract.restype = i
        L.qto_net_lg_wire_ids.argtypes = [ctypes.c_void_p, P(i), P(i), P(i), i]
        L.qto_net_lg_wire_ids.restype = i
        L.qto_net_final_value.argtypes = [ctypes.c_void_p, P(d)]
        L.qto_net_final_value.restype = None
        L.qto_net_flops.argtypes = [ctypes.c_void_p]
        L.qto_net_flops.restype = ctypes.c_int64
        L.qto_net_created_from.argtypes = [ctypes.c_void_p, P(i), i]
        L.qto_net_created_from.restype = i
        L.qto_net_remaining_value.argtypes = [ctypes.c_void_p, P(d)]
        L.qto_net_remaining_value.restype = i
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def contract_indices(a, b, free_from_a, free_idx, sum_a, sum_b):
    """One ContractIndices call on complex128 numpy vectors (flat base-4 layout)."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    ra = int(round(np.log(a.size) / np.log(4))) if a.size > 1 else 0
    rb = int(round(np.log(b.size) / np.log(4))) if b.size > 1 else 0
    nf = len(free_idx)
    c = np.zeros(4 ** nf, dtype=np.complex128)
    ffa = np.ascontiguousarray(free_from_a, dtype=np.int32)
    fi = np.ascontiguousarray(free_idx, dtype=np.int32)
    sa = np.ascontiguousarray(sum_a, dtype=np.int32)
    sb = np.ascontiguousarray(sum_b, dtype=np.int32)
    lib().qto_contract_indices(ra, _dp(a.view(np.float64)), rb, _dp(b.view(np.float64)), nf, _ip(ffa), _ip(fi),
                               len(sum_a), _ip(sa), _ip(sb), _dp(c.view(np.float64)))
    return c


def gate_tensor(name, param=0.0):
    out = np.zeros(256, dtype=np.complex128)
    r = lib().qto_gate_tensor(name.encode(), float(param), _dp(out.view(np.float64)))
    if r < 0:
        raise OracleError(QTO_INVALID_FUNCTION_INPUT, name)
    return out[: 4 ** r].copy()


def arbitrary_gate(path, two_qubit):
    out = np.zeros(256, dtype=np.complex128)
    r = lib().qto_arbitrary_gate(path.encode(), 1 if two_qubit else 0, _dp(out.view(np.float64)))
    if r < 0:
        raise OracleError(-r, path)
    return out[: 4 ** r].copy()


class Net:
    """A parsed network of the oracle port (mirrors Network's observable state)."""

    def __init__(self, qasm_text, measure_text="", gate_dir=None):
        err = ctypes.c_int(0)
        self._h = lib().qto_net_parse(qasm_text.encode(), measure_text.encode(),
                                      gate_dir.encode() if gate_dir else None, ctypes.byref(err))
        if not self._h:
            raise OracleError(err.value, "parse")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.qto_net_free(h)
            self._h = None

    @property
    def num_nodes(self):
        return lib().qto_net_num_nodes(self._h)

    @property
    def num_qubits(self):
        return lib().qto_net_num_qubits(self._h)

    def node_rank(self, i):
        return lib().qto_net_node_rank(self._h, i)

    def node_values(self, i):
        r = self.node_rank(i)
        out = np.zeros(4 ** r, dtype=np.complex128)
        ok = lib().qto_net_node_values(self._h, i, _dp(out.view(np.float64)), 2 * out.size)
        return out if ok == 1 else None

    def contract(self, a, b, threshold):
        return lib().qto_net_contract(self._h, a, b, threshold)

    def replay(self, pairs):
        arr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1))
        rc = lib().qto_net_replay(self._h, _ip(arr), arr.size // 2)
        if rc != QTO_OK:
            raise OracleError(rc, "replay")

    def lg_contract(self, order_1based):
        arr = np.ascontiguousarray(np.asarray(order_1based, dtype=np.int32))
        rc = lib().qto_net_lg_contract(self._h, _ip(arr), arr.size)
        if rc != QTO_OK:
            raise OracleError(rc, "lg_contract")

    def lg_wire_ids(self):
        n = self.num_nodes
        nodes = np.zeros(n, dtype=np.int32)
        ranks = np.zeros(n, dtype=np.int32)
        wires = np.zeros(64 * n + 64, dtype=np.int32)
        lib().qto_net_lg_wire_ids(self._h, _ip(nodes), _ip(ranks), _ip(wires), wires.size)
        out, pos = [], 0
        for k in range(n):
            out.append((int(nodes[k]), [int(x) for x in wires[pos: pos + ranks[k]]]))
            pos += ranks[k]
        return out

    @property
    def done(self):
        return bool(lib().qto_net_done(self._h))

    @property
    def final_value(self):
        v = np.zeros(2)
        lib().qto_net_final_value(self._h, _dp(v))
        return complex(v[0], v[1])

    @property
    def remaining_value(self):
        v = np.zeros(2)
        rc = lib().qto_net_remaining_value(self._h, _dp(v))
        if rc != QTO_OK:
            raise OracleError(rc, "remaining")
        return complex(v[0], v[1])

    @property
    def flops(self):
        return int(lib().qto_net_flops(self._h))

    def created_from(self):
        cap = 4 * self.num_nodes + 16
        arr = np.zeros(2 * cap, dtype=np.int32)
        n = lib().qto_net_created_from(self._h, _ip(arr), cap)
        return [(int(arr[2 * i]), int(arr[2 * i + 1])) for i in range(n)]


def replay_value(qasm_text, measure_text, pairs, gate_dir=None):
    net = Net(qasm_text, measure_text, gate_dir)
    net.replay(pairs)
    return net.final_value, net.flops
