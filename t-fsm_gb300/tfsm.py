"""ctypes binding of the C ABI in include/tfsm.h (libtfsm_gb300.so in this directory).

The library is the product path: there is no Python or CPU fallback.  Loading fails loudly when
the shared library has not been built (run t-fsm_gb300/build.py) and every call that fails raises
TfsmError with the library's message.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path
from typing import Iterable, Sequence

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libtfsm_gb300.so"

TFSM_OK = 0
TFSM_ERR_ARG = 1
TFSM_ERR_IO = 2
TFSM_ERR_FORMAT = 3
TFSM_ERR_PATTERN = 4
TFSM_ERR_LIMIT = 5
TFSM_ERR_NO_DEVICE = 9
TFSM_ERR_CUDA = 10
TFSM_ERR_INTERNAL = 11
MAX_PATTERN_VERTICES = 32
MAX_LEVELS = 32

FLAG_EXACT = 1
FLAG_PLAIN = 2
FLAG_NO_SPLIT = 4
FLAG_NO_SUBPATTERN_PRUNING = 8

EXPORTED = (
    "tfsm_graph_load",
    "tfsm_graph_from_edges",
    "tfsm_graph_free",
    "tfsm_graph_info",
    "tfsm_graph_export",
    "tfsm_evaluate_support",
    "tfsm_evaluate_batch",
    "tfsm_evaluate_level",
    "tfsm_domains_free",
    "tfsm_mine",
    "tfsm_get_options",
    "tfsm_set_options",
    "tfsm_set_level_options",
    "tfsm_evaluate_support_noalloc",
    "tfsm_cost_model_create",
    "tfsm_cost_model_free",
    "tfsm_cost_model_get_params",
    "tfsm_cost_model_set_params",
    "tfsm_cost_model_predict",
    "tfsm_cost_model_gradients",
    "tfsm_cost_model_train",
    "tfsm_set_order_policy",
    "tfsm_record_orders",
    "tfsm_take_records",
    "tfsm_last_error",
)

COST_FEATURES = 32
COST_PARAMS = 6337
ORDER_GQL, ORDER_RANDOM, ORDER_MODEL = 0, 1, 2


class TfsmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tfsm error {code}: {msg}")
        self.code = code


class DfsCode(C.Structure):
    _fields_ = [("from_", C.c_int32), ("to", C.c_int32), ("from_label", C.c_int32), ("edge_label", C.c_int32),
                ("to_label", C.c_int32)]


class PatternC(C.Structure):
    _fields_ = [("n_codes", C.c_int32), ("codes", C.POINTER(DfsCode))]


class ParentC(C.Structure):
    _fields_ = [("domains", C.c_void_p), ("index", C.c_int32)]


class ResultC(C.Structure):
    _fields_ = [("status", C.c_int32), ("frequent", C.c_int32), ("n_vertices", C.c_int32),
                ("decided_by_filter", C.c_int32), ("support", C.c_uint32),
                ("mni", C.c_uint32 * MAX_PATTERN_VERTICES), ("searches", C.c_uint64), ("steps", C.c_uint64)]


class GraphInfoC(C.Structure):
    _fields_ = [("n_vertices", C.c_uint32), ("n_edges", C.c_uint64), ("n_frequent_vertex_labels", C.c_uint32),
                ("n_frequent_edge_labels", C.c_uint32), ("n_frequent_edge_patterns", C.c_uint32),
                ("max_degree", C.c_uint32), ("device_bytes", C.c_uint64), ("load_ms", C.c_double),
                ("load_h2d_bytes", C.c_uint64)]


class EdgePatternC(C.Structure):
    _fields_ = [("la", C.c_int32), ("el", C.c_int32), ("lb", C.c_int32), ("cand_a", C.c_uint32),
                ("cand_b", C.c_uint32)]


class GraphArraysC(C.Structure):
    _fields_ = [("row_off", C.c_void_p), ("col", C.c_void_p), ("elab", C.c_void_p), ("label_start", C.c_void_p),
                ("lab_off", C.c_void_p), ("vlabels", C.c_void_p), ("elabels", C.c_void_p),
                ("edge_patterns", C.c_void_p), ("label_mean_degree", C.c_void_p)]


class OptionsC(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("step_budget", C.c_uint32), ("split_slice", C.c_uint32),
                ("chunk_words", C.c_uint32), ("refine_rounds", C.c_uint32), ("max_batch", C.c_uint32),
                ("hub_span", C.c_uint32), ("hub_parts", C.c_uint32), ("time_limit_s", C.c_double),
                ("search_lanes", C.c_uint32), ("rank_window", C.c_uint32), ("call_ms", C.c_double),
                ("isect_ratio", C.c_uint32), ("reserved", C.c_uint32), ("refine_scope", C.c_uint32),
                ("reserved2", C.c_uint32)]

    def __init__(self, **kw):
        super().__init__(**kw)
        self.struct_size = C.sizeof(OptionsC)


class MineStatsC(C.Structure):
    _fields_ = [("load_ms", C.c_double), ("mine_ms", C.c_double), ("extend_ms", C.c_double),
                ("init_ms", C.c_double), ("refine_ms", C.c_double), ("search_ms", C.c_double),
                ("init_launches", C.c_uint64), ("refine_launches", C.c_uint64), ("search_launches", C.c_uint64),
                ("init_words", C.c_uint64), ("refine_words", C.c_uint64), ("search_bytes", C.c_uint64),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("evaluations", C.c_uint64), ("frequent", C.c_uint64), ("searches", C.c_uint64),
                ("steps", C.c_uint64), ("by_filter", C.c_uint64), ("engine_calls", C.c_uint64),
                ("levels", C.c_int32), ("complete", C.c_int32), ("level_ms", C.c_double * MAX_LEVELS),
                ("pruned", C.c_uint64), ("split_searches", C.c_uint64), ("split_tasks", C.c_uint64),
                ("intersections", C.c_uint64)]


_lib = None


def lib() -> C.CDLL:
    """The loaded C library (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(f"{LIB_PATH} is missing: build it with t-fsm_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        L.tfsm_graph_load.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]
        L.tfsm_graph_from_edges.argtypes = [C.c_uint32, C.POINTER(C.c_int32), C.c_uint64, C.POINTER(C.c_uint32),
                                            C.POINTER(C.c_uint32), C.POINTER(C.c_int32), C.c_int32,
                                            C.POINTER(C.c_void_p)]
        L.tfsm_graph_free.argtypes = [C.c_void_p]
        L.tfsm_graph_free.restype = None
        L.tfsm_graph_info.argtypes = [C.c_void_p, C.POINTER(GraphInfoC)]
        L.tfsm_graph_export.argtypes = [C.c_void_p, C.POINTER(GraphArraysC)]
        L.tfsm_evaluate_support.argtypes = [C.c_void_p, C.POINTER(PatternC), C.c_int32, C.c_uint32,
                                            C.POINTER(ResultC)]
        L.tfsm_evaluate_batch.argtypes = [C.c_void_p, C.POINTER(PatternC), C.c_int32, C.c_int32, C.c_uint32,
                                          C.POINTER(ResultC)]
        L.tfsm_evaluate_level.argtypes = [C.c_void_p, C.POINTER(PatternC), C.c_int32, C.c_int32, C.c_uint32,
                                          C.POINTER(ParentC), C.POINTER(ResultC), C.POINTER(C.c_void_p)]
        L.tfsm_domains_free.argtypes = [C.c_void_p]
        L.tfsm_domains_free.restype = None
        L.tfsm_mine.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_uint32, C.c_char_p, C.POINTER(MineStatsC)]
        L.tfsm_get_options.argtypes = [C.c_void_p, C.POINTER(OptionsC)]
        L.tfsm_set_options.argtypes = [C.c_void_p, C.POINTER(OptionsC)]
        L.tfsm_set_level_options.argtypes = [C.c_void_p, C.c_int32, C.POINTER(OptionsC)]
        L.tfsm_evaluate_support_noalloc.argtypes = [C.c_void_p, C.POINTER(PatternC), C.c_int32, C.c_uint32,
                                                    C.POINTER(ResultC)]
        fp = C.POINTER(C.c_float)
        L.tfsm_cost_model_create.argtypes = [C.c_uint64, C.POINTER(C.c_void_p)]
        L.tfsm_cost_model_free.argtypes = [C.c_void_p]
        L.tfsm_cost_model_free.restype = None
        L.tfsm_cost_model_get_params.argtypes = [C.c_void_p, fp]
        L.tfsm_cost_model_set_params.argtypes = [C.c_void_p, fp]
        L.tfsm_cost_model_predict.argtypes = [C.c_void_p, fp, C.c_uint64, fp]
        L.tfsm_cost_model_gradients.argtypes = [C.c_void_p, fp, fp, C.c_uint64, fp]
        L.tfsm_cost_model_train.argtypes = [C.c_void_p, fp, fp, C.c_uint64, C.c_int32, C.c_int32, C.c_float,
                                            C.c_uint64, C.POINTER(C.c_double)]
        L.tfsm_set_order_policy.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_void_p]
        L.tfsm_record_orders.argtypes = [C.c_void_p, C.c_int32]
        L.tfsm_take_records.argtypes = [C.c_void_p, fp, fp, C.c_uint64, C.POINTER(C.c_uint64)]
        L.tfsm_last_error.argtypes = []
        L.tfsm_last_error.restype = C.c_char_p
        for f in EXPORTED:
            if f not in ("tfsm_graph_free", "tfsm_last_error", "tfsm_cost_model_free", "tfsm_domains_free"):
                getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != TFSM_OK:
        raise TfsmError(rc, lib().tfsm_last_error().decode(errors="replace"))


Code = tuple  # (from, to, from_label, edge_label, to_label)


def parse_key(key: str) -> list[Code]:
    """'0,1,3,1,4 1,2,4,1,4' -> [(0,1,3,1,4), (1,2,4,1,4)]"""
    return [tuple(int(x) for x in tok.split(",")) for tok in key.split()]


def make_key(codes: Sequence[Code]) -> str:
    return " ".join(",".join(str(x) for x in c) for c in codes)


@dataclass
class Result:
    status: int
    frequent: bool
    support: int
    mni: list
    decided_by_filter: bool
    searches: int
    steps: int


def _pattern_array(patterns: Iterable[Sequence[Code]]):
    pats = [list(p) for p in patterns]
    n = len(pats)
    keep = []
    arr = (PatternC * max(n, 1))()
    for i, p in enumerate(pats):
        codes = (DfsCode * max(len(p), 1))(*[DfsCode(*c) for c in p])
        keep.append(codes)
        arr[i].n_codes = len(p)
        arr[i].codes = C.cast(codes, C.POINTER(DfsCode))
    return arr, n, keep


def _results(res, n: int) -> list[Result]:
    return [Result(r.status, bool(r.frequent), r.support, list(r.mni[: r.n_vertices]), bool(r.decided_by_filter),
                   r.searches, r.steps) for r in res[:n]]


class Domains:
    """Final domains of one Graph.evaluate_level call, kept on the device (tfsm_domains)."""

    def __init__(self, h: int):
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().tfsm_domains_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown: the library may already be gone
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Graph:
    """A pruned data graph resident on the GPU (tfsm_graph)."""

    def __init__(self, handle: C.c_void_p, tau: int):
        self._h = handle
        self.tau = tau

    @classmethod
    def load(cls, path: str | Path, tau: int) -> "Graph":
        h = C.c_void_p()
        _check(lib().tfsm_graph_load(str(path).encode(), int(tau), C.byref(h)))
        return cls(h, tau)

    @classmethod
    def from_edges(cls, vlabels, src, dst, elabels, tau: int) -> "Graph":
        import numpy as np

        vl = np.ascontiguousarray(vlabels, dtype=np.int32)
        s = np.ascontiguousarray(src, dtype=np.uint32)
        d = np.ascontiguousarray(dst, dtype=np.uint32)
        el = np.ascontiguousarray(elabels, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().tfsm_graph_from_edges(
            len(vl), vl.ctypes.data_as(C.POINTER(C.c_int32)), len(s), s.ctypes.data_as(C.POINTER(C.c_uint32)),
            d.ctypes.data_as(C.POINTER(C.c_uint32)), el.ctypes.data_as(C.POINTER(C.c_int32)), int(tau),
            C.byref(h)))
        return cls(h, tau)

    def close(self) -> None:
        if self._h:
            lib().tfsm_graph_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        gi = GraphInfoC()
        _check(lib().tfsm_graph_info(self._h, C.byref(gi)))
        return {f: getattr(gi, f) for f, _ in GraphInfoC._fields_}

    def export(self) -> dict:
        """The graph as the device holds it (tfsm_graph_export): numpy arrays row_off, col, elab,
        label_start, lab_off, vlabels, elabels, label_mean_degree, and edge_patterns as a list of
        (la, el, lb, cand_a, cand_b)."""
        import numpy as np

        gi = self.info()
        n, m2 = gi["n_vertices"], 2 * gi["n_edges"]
        nl, ne, npat = gi["n_frequent_vertex_labels"], gi["n_frequent_edge_labels"], gi["n_frequent_edge_patterns"]
        out = dict(row_off=np.zeros(n + 1, np.uint32), col=np.zeros(m2, np.uint32), elab=np.zeros(m2, np.uint8),
                   label_start=np.zeros(nl + 1, np.uint32), lab_off=np.zeros(n * (nl + 1), np.uint32),
                   vlabels=np.zeros(nl, np.int32), elabels=np.zeros(ne, np.int32),
                   label_mean_degree=np.zeros(nl, np.float32))
        pats = (EdgePatternC * max(npat, 1))()
        a = GraphArraysC(**{k: v.ctypes.data for k, v in out.items()}, edge_patterns=C.cast(pats, C.c_void_p))
        _check(lib().tfsm_graph_export(self._h, C.byref(a)))
        out["edge_patterns"] = [(p.la, p.el, p.lb, p.cand_a, p.cand_b) for p in pats[:npat]]
        return out

    def evaluate(self, patterns: Iterable[Sequence[Code]], tau: int | None = None, flags: int = 0) -> list[Result]:
        arr, n, _keep = _pattern_array(patterns)
        res = (ResultC * max(n, 1))()
        rc = lib().tfsm_evaluate_batch(self._h, arr, n, int(self.tau if tau is None else tau), int(flags), res)
        _check(rc)
        return _results(res, n)

    def evaluate_level(self, patterns: Iterable[Sequence[Code]], parents: Sequence | None = None,
                       tau: int | None = None, flags: int = 0, keep: bool = False):
        """tfsm_evaluate_level: like evaluate, with parents[i] = (Domains, index) or None per pattern.
        Returns (results, Domains or None); with keep=True the call's final domains stay on the
        device for the next level's parents."""
        arr, n, _keep = _pattern_array(patterns)
        par = None
        if parents is not None:
            if len(parents) != n:
                raise ValueError("one parent entry per pattern")
            par = (ParentC * max(n, 1))()
            for i, pr in enumerate(parents):
                if pr is not None:
                    d, idx = pr
                    par[i].domains = d._h
                    par[i].index = int(idx)
        res = (ResultC * max(n, 1))()
        h = C.c_void_p()
        rc = lib().tfsm_evaluate_level(self._h, arr, n, int(self.tau if tau is None else tau), int(flags), par, res,
                                       C.byref(h) if keep else None)
        _check(rc)
        return _results(res, n), (Domains(h.value) if keep and h.value else None)

    def options(self) -> dict:
        o = OptionsC()
        _check(lib().tfsm_get_options(self._h, C.byref(o)))
        return {f: getattr(o, f) for f, _ in OptionsC._fields_ if f not in ("struct_size", "reserved", "reserved2")}

    def set_options(self, **kw) -> None:
        cur = self.options()
        cur.update(kw)
        o = OptionsC(**cur)
        _check(lib().tfsm_set_options(self._h, C.byref(o)))

    def set_level_options(self, level: int, options: dict | None) -> None:
        """Knobs for the engine calls of one growth level (patterns with `level` edges); None clears
        the level, level 0 clears all.  Missing keys take the handle's current options."""
        if options is None:
            _check(lib().tfsm_set_level_options(self._h, level, None))
            return
        cur = self.options()
        cur.update(options)
        o = OptionsC(**cur)
        _check(lib().tfsm_set_level_options(self._h, level, C.byref(o)))

    def set_order_policy(self, policy: int, seed: int = 0, model: "CostModel | None" = None) -> None:
        self._model = model  # kept alive while the handle may use it
        _check(lib().tfsm_set_order_policy(self._h, policy, seed, model._h if model else None))

    def record_orders(self, enable: bool = True) -> None:
        _check(lib().tfsm_record_orders(self._h, 1 if enable else 0))

    def take_records(self):
        """(features [n x 32] float32, costs [n] float32) recorded so far; clears them."""
        import numpy as np

        n = C.c_uint64(0)
        _check(lib().tfsm_take_records(self._h, None, None, 0, C.byref(n)))
        f = np.zeros((n.value, COST_FEATURES), dtype=np.float32)
        c = np.zeros(n.value, dtype=np.float32)
        got = C.c_uint64(0)
        _check(lib().tfsm_take_records(self._h, _fptr(f), _fptr(c), n.value, C.byref(got)))
        return f[: got.value], c[: got.value]

    def mine(self, max_nodes: int = -1, flags: int = 0, results_path: str | Path | None = None,
             tau: int | None = None) -> dict:
        st = MineStatsC()
        p = str(results_path).encode() if results_path else None
        _check(lib().tfsm_mine(self._h, int(self.tau if tau is None else tau), int(max_nodes), int(flags), p,
                               C.byref(st)))
        return {f: (list(getattr(st, f)) if f == "level_ms" else getattr(st, f)) for f, _ in MineStatsC._fields_}


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class CostModel:
    """The learned matching-order cost model (32-64-64-1 MLP, BF16 weights, trained on the GPU)."""

    def __init__(self, seed: int = 0):
        h = C.c_void_p()
        _check(lib().tfsm_cost_model_create(seed, C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().tfsm_cost_model_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        import numpy as np

        p = np.zeros(COST_PARAMS, dtype=np.float32)
        _check(lib().tfsm_cost_model_get_params(self._h, _fptr(p)))
        return p

    def set_params(self, p) -> None:
        import numpy as np

        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (COST_PARAMS,)
        _check(lib().tfsm_cost_model_set_params(self._h, _fptr(p)))

    def predict(self, x):
        import numpy as np

        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, COST_FEATURES)
        y = np.zeros(len(x), dtype=np.float32)
        _check(lib().tfsm_cost_model_predict(self._h, _fptr(x), len(x), _fptr(y)))
        return y

    def gradients(self, x, t):
        import numpy as np

        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, COST_FEATURES)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.zeros(COST_PARAMS, dtype=np.float32)
        _check(lib().tfsm_cost_model_gradients(self._h, _fptr(x), _fptr(t), len(x), _fptr(g)))
        return g

    def train(self, x, t, epochs: int = 20, batch: int = 256, lr: float = 1e-3, seed: int = 0) -> float:
        import numpy as np

        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, COST_FEATURES)
        t = np.ascontiguousarray(t, dtype=np.float32)
        mse = C.c_double(0)
        _check(lib().tfsm_cost_model_train(self._h, _fptr(x), _fptr(t), len(x), epochs, batch, lr, seed,
                                           C.byref(mse)))
        return mse.value


def read_results(path: str | Path) -> list[str]:
    """Pattern keys of a grami_results.txt file (serial reference format), in file order."""
    pats, cur_v, cur_e = [], [], []

    def flush():
        if cur_v:
            pats.append(" ".join(f"{a},{b},{cur_v[a]},{l},{cur_v[b]}" for a, b, l in cur_e))

    for line in Path(path).read_text().splitlines():
        t = line.split()
        if not t:
            continue
        if t[0].startswith("====="):
            flush()
            cur_v, cur_e = [], []
        elif t[0] == "v":
            cur_v.append(int(t[2]))
        elif t[0] == "e":
            cur_e.append((int(t[1]), int(t[2]), int(t[3])))
    flush()
    return pats
