"""ctypes binding of include/fem_tet.h (libfemtet_gb300.so).

The library is loaded from this package directory only; there is no other
implementation behind these calls. If the shared library is missing or has
no usable CUDA device, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# FEMGB_BOUNDS_CHECK=1 selects the diagnostic build whose kernels check every
# table-read index (build.build_bounds_check()); otherwise the normal library.
BOUNDS_LIB_PATH = os.path.join(HERE, "libfemtet_gb300_bounds.so")
LIB_PATH = BOUNDS_LIB_PATH if os.environ.get("FEMGB_BOUNDS_CHECK") == "1" else os.path.join(HERE, "libfemtet_gb300.so")
# FEMGB_LIBRARY names another build of the same library (a variant compiled
# with other -D settings by build.build(defines=..., out=...)).
LIB_PATH = os.environ.get("FEMGB_LIBRARY") or LIB_PATH

FEM_OK = 0
FEM_E_ARG, FEM_E_INDEX, FEM_E_NAN, FEM_E_OOM, FEM_E_CUDA, FEM_E_TIMEOUT, FEM_E_NODEVICE, FEM_E_DEGENERATE = range(1, 9)
FEM_PRECISION_FP64 = 0
FEM_PRECISION_MIXED = 1
FEM_INTEGRATOR_QIE_V = 0
FEM_INTEGRATOR_FIE_DX = 1
FEM_INTEGRATOR_FIE_DX_QUASISTATIC = 2
FEM_ROTATION_MSVD = 0
FEM_ROTATION_DAPD = 1
FEM_LS_CG = 0
FEM_LS_MINRES = 1
FEM_MATERIAL_C_WRP = 0
FEM_MATERIAL_C_LCM = 1
FEM_MATERIAL_C_LCMH = 2
FEM_MATERIAL_C_CCM = 3
FEM_WAIT_LIMIT_DEFAULT = 0xFFFFFFFF

_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)


class FemParams(C.Structure):
    _fields_ = [
        ("fixed_dt", C.c_double),
        ("density", C.c_double),
        ("young_modulus", C.c_double),
        ("poisson_ratio", C.c_double),
        ("damping_ratio", C.c_double),
        ("gravity", C.c_double * 3),
        ("ls_rel_epsilon", C.c_double),
        ("ls_abs_epsilon", C.c_double),
        ("ls_max_iter", C.c_uint32),
        ("precision", C.c_uint32),
        ("degenerate_det_F", C.c_double),
        ("refresh_every", C.c_uint32),
        ("compute_energy", C.c_uint32),
        ("rotation_check", C.c_double),
        ("refresh_drop", C.c_double),
        ("rotation_fp32", C.c_uint32),
        ("integrator", C.c_uint32),
        ("nr_max_iter", C.c_uint32),
        ("rotation", C.c_uint32),
        ("ls_solver", C.c_uint32),
        ("nr_abs_epsilon", C.c_double),
        ("dapd_threshold_det_F", C.c_double),
        ("dapd_l_factor", C.c_double),
        ("dapd_nl_factor", C.c_double),
        ("dapd_nl_exponent", C.c_double),
        ("material", C.c_uint32),
        ("pad", C.c_uint32),
        ("ecie_k_factor", C.c_double),
    ]


class FemStepStats(C.Structure):
    _fields_ = [
        ("cg_iterations", C.c_uint32),
        ("status", C.c_uint32),
        ("rel_residual", C.c_double),
        ("abs_residual", C.c_double),
        ("elastic_energy", C.c_double),
        ("potential_energy", C.c_double),
        ("inverted_elements", C.c_uint32),
        ("fp64_resolved", C.c_uint32),
        ("total_cg_iterations", C.c_uint64),
        ("nr_iterations", C.c_uint32),
        ("pad", C.c_uint32),
        ("nr_rel_residual", C.c_double),
        ("nr_abs_residual", C.c_double),
        ("resolved_det_F", C.c_uint32),
        ("resolved_isotropic", C.c_uint32),
        ("resolved_tie", C.c_uint32),
        ("resolved_check", C.c_uint32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


class FemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fem status {code}: {msg}")
        self.code = code


# Every exported symbol of include/fem_tet.h with its ctypes signature.
SIGNATURES = {
    "fem_params_default": (C.c_int, [C.POINTER(FemParams)]),
    "fem_solid_create": (C.c_int, [_dp, C.c_uint32, _up, C.c_uint32, C.POINTER(FemParams), _dp, _dp,
                                   C.POINTER(C.c_void_p)]),
    "fem_solid_destroy": (C.c_int, [C.c_void_p]),
    "fem_solid_get_sizes": (C.c_int, [C.c_void_p, _up, _up]),
    "fem_solid_set_knc": (C.c_int, [C.c_void_p, _up, _dp, C.c_uint32]),
    "fem_solid_set_knc_targets": (C.c_int, [C.c_void_p, _dp]),
    "fem_solid_set_state": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fem_solid_get_state": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fem_solid_step": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(FemStepStats)]),
    "fem_solid_step_host": (C.c_int, [C.c_void_p, _dp, _dp, C.c_uint32, _dp, _dp, C.POINTER(FemStepStats)]),
    "fem_solid_begin_eval": (C.c_int, [C.c_void_p, _dp]),
    "fem_solid_get_rotations": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fem_solid_get_doc": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8)]),
    "fem_tetgen_read": (C.c_int, [C.c_char_p, C.c_char_p, C.c_double, _dp, C.c_uint32, _up, C.c_uint32, _up, _up,
                                  _up]),
    "fem_tetshape_rebuild": (C.c_int, [_dp, C.c_uint32, _up, C.c_uint32, _dp, _up, _up, _up, _up, _up, _up,
                                       C.c_uint32, _up, _up, C.c_uint32, _up]),
    "fem_geo_write": (C.c_int, [C.c_char_p, _dp, C.c_uint32, _up, C.c_uint32]),
    "fem_geo_read": (C.c_int, [C.c_char_p, _dp, C.c_uint32, _up, C.c_uint32, _up, _up, _up]),
    "fem_tetgen_to_geo": (C.c_int, [C.c_char_p, C.c_char_p, C.c_double, C.c_char_p]),
    "fem_solid_force_elastic": (C.c_int, [C.c_void_p, _dp]),
    "fem_solid_df_x": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fem_solid_apply_A": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _dp, _dp]),
    "fem_solid_energy": (C.c_int, [C.c_void_p, _dp]),
    "fem_solid_mass_info": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "fem_solid_apply_A_noalloc": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _dp, _dp]),
    "fem_solid_set_params": (C.c_int, [C.c_void_p, C.POINTER(FemParams)]),
    "fem_solid_set_assembled": (C.c_int, [C.c_void_p, C.c_int]),
    "fem_solid_nr_init": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_solid_nr_prestep": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_solid_nr_midstep": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_solid_nr_poststep": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_solid_nr_end": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_multi_step": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.c_double, C.c_uint32]),
    "fem_solid_get_params": (C.c_int, [C.c_void_p, C.POINTER(FemParams)]),
    "fem_solid_get_dapd_state": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_uint8)]),
    "fem_solid_set_dapd_state": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_uint8)]),
    "fem_solid_step_async": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fem_solid_synchronize": (C.c_int, [C.c_void_p, C.POINTER(FemStepStats)]),
    "fem_solid_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "fem_last_error": (C.c_char_p, []),
    "fem_device_info": (C.c_int, [C.POINTER(C.c_int)] * 4),
    "fem_kernel_launches": (C.c_uint64, []),
    "fem_profile_enable": (C.c_int, [C.c_int]),
    "fem_profile_read": (C.c_int, [C.c_char_p, _dp, C.POINTER(C.c_ulonglong)]),
    "fem_bounds_check_status": (C.c_int, [C.POINTER(C.c_int)] + [_up] * 4),
}

_lib = None


def load():
    """Load libfemtet_gb300.so from the package directory (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    _bind_batch_signatures()
    if not os.path.exists(LIB_PATH):
        raise FemError(FEM_E_NODEVICE, f"{LIB_PATH} is missing: run __graft_entry__.build()")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code):
    if code != FEM_OK:
        raise FemError(code, load().fem_last_error().decode(errors="replace"))


def _ptr(a, ctype=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(ctype))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def default_params() -> FemParams:
    p = FemParams()
    check(load().fem_params_default(C.byref(p)))
    return p


def params_for(scene, precision: int = FEM_PRECISION_FP64, compute_energy: bool = True) -> FemParams:
    p = default_params()
    p.fixed_dt = scene.dt
    p.density = scene.density
    p.young_modulus = scene.young
    p.poisson_ratio = scene.poisson
    p.damping_ratio = scene.damping_ratio
    for i in range(3):
        p.gravity[i] = scene.gravity[i]
    p.ls_rel_epsilon = scene.rel_eps
    p.ls_abs_epsilon = scene.abs_eps
    p.ls_max_iter = scene.max_iter
    p.precision = precision
    p.compute_energy = 1 if compute_energy else 0
    p.integrator = getattr(scene, "integrator", FEM_INTEGRATOR_QIE_V)
    p.nr_max_iter = getattr(scene, "nr_max_iter", 3)
    p.nr_abs_epsilon = getattr(scene, "nr_abs_eps", 1e-6)
    p.ls_solver = getattr(scene, "ls_solver", FEM_LS_CG)
    p.material = getattr(scene, "material", FEM_MATERIAL_C_WRP)
    p.ecie_k_factor = getattr(scene, "ecie_k_factor", 1.0)
    p.rotation = getattr(scene, "rotation", FEM_ROTATION_MSVD)
    if p.rotation == FEM_ROTATION_DAPD:
        p.dapd_threshold_det_F = scene.dapd_threshold
        p.dapd_l_factor = scene.dapd_L
        p.dapd_nl_factor = scene.dapd_NL
        p.dapd_nl_exponent = scene.dapd_exponent
    return p


class Solid:
    """One device-resident solid (the Solid3D / LeafDSH_Solid3D_FEM seam)."""

    def __init__(self, scene, precision: int = FEM_PRECISION_FP64, compute_energy: bool = True,
                 params: Optional[FemParams] = None):
        lib = load()
        self.lib = lib
        self.scene = scene
        self.N = scene.num_nodes
        self.T = scene.num_tets
        self.params = params if params is not None else params_for(scene, precision, compute_energy)
        rest = _f64(scene.rest)
        tets = np.ascontiguousarray(scene.tets, dtype=np.uint32)
        Ep = _f64(scene.young_per_elem)
        nup = _f64(scene.poisson_per_elem)
        h = C.c_void_p()
        check(lib.fem_solid_create(_ptr(rest), self.N, _ptr(tets, C.c_uint32), self.T, C.byref(self.params),
                                   _ptr(Ep), _ptr(nup), C.byref(h)))
        self.h = h
        self._knc_nodes = np.ascontiguousarray(scene.knc_nodes, dtype=np.uint32)
        if self._knc_nodes.size:
            tg = _f64(scene.targets_at(0) if scene.knc_schedule is not None else scene.knc_targets)
            check(lib.fem_solid_set_knc(h, _ptr(self._knc_nodes, C.c_uint32), _ptr(tg), self._knc_nodes.size))
        if scene.init_vel is not None:
            self.set_state(v=scene.init_vel)
        self.step_index = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.fem_solid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, x=None, v=None):
        x, v = _f64(x), _f64(v)
        check(self.lib.fem_solid_set_state(self.h, _ptr(x), _ptr(v)))

    def state(self):
        x = np.empty((self.N, 3))
        v = np.empty((self.N, 3))
        check(self.lib.fem_solid_get_state(self.h, _ptr(x), _ptr(v)))
        return x, v

    def set_knc_targets(self, targets):
        t = _f64(targets)
        check(self.lib.fem_solid_set_knc_targets(self.h, _ptr(t)))

    def set_params(self, params):
        """Run-time parameter change (fem_solid_set_params)."""
        check(self.lib.fem_solid_set_params(self.h, C.byref(params)))
        self.params = params

    def get_params(self):
        p = FemParams()
        check(self.lib.fem_solid_get_params(self.h, C.byref(p)))
        return p

    def set_assembled(self, on: bool = True):
        """fem_solid_set_assembled: the solvers take K u from an assembled
        3x3-block stiffness (on) or from the element products (off, the
        default)."""
        check(self.lib.fem_solid_set_assembled(self.h, 1 if on else 0))

    def nr_phase(self, phase, dt):
        """One multi-solid Newton lock-step phase (init, prestep, midstep,
        poststep, end; fem_solid_nr_*)."""
        check(getattr(self.lib, "fem_solid_nr_" + phase)(self.h, float(dt)))

    def stats(self):
        st = FemStepStats()
        check(self.lib.fem_solid_synchronize(self.h, C.byref(st)))
        return st.as_dict()

    def dapd_state(self):
        """(previous positions (N, 3), directions of collapse (T, 2))."""
        px = np.empty((self.N, 3))
        doc = np.empty((self.T, 2), np.uint8)
        check(self.lib.fem_solid_get_dapd_state(self.h, _ptr(px), doc.ctypes.data_as(C.POINTER(C.c_uint8))))
        return px, doc

    def set_dapd_state(self, prev_x=None, doc=None):
        px = _f64(prev_x)
        d = None if doc is None else np.ascontiguousarray(doc, dtype=np.uint8)
        check(self.lib.fem_solid_set_dapd_state(self.h, _ptr(px),
                                                None if d is None else d.ctypes.data_as(C.POINTER(C.c_uint8))))

    def step(self, n: int = 1):
        st = FemStepStats()
        sc = self.scene
        if sc.knc_schedule is not None and self._knc_nodes.size:
            out = []
            for _ in range(n):
                self.set_knc_targets(sc.targets_at(self.step_index))
                check(self.lib.fem_solid_step(self.h, 1, C.byref(st)))
                self.step_index += 1
                out.append(st.as_dict())
            return out[-1]
        check(self.lib.fem_solid_step(self.h, n, C.byref(st)))
        self.step_index += n
        return st.as_dict()

    def run(self, steps=None):
        steps = self.scene.steps if steps is None else steps
        return [self.step(1) for _ in range(steps)]

    # ---- element-level hooks ----
    def begin_eval(self, x):
        x = _f64(x)
        check(self.lib.fem_solid_begin_eval(self.h, _ptr(x)))

    def rotations(self):
        R = np.empty((self.T, 3, 3))
        d = np.empty(self.T)
        check(self.lib.fem_solid_get_rotations(self.h, _ptr(R), _ptr(d)))
        return R, d

    def doc(self):
        """DAPD: per-element direction of collapse (vit0, vit1); (3, 0) = none."""
        d = np.empty((self.T, 2), np.uint8)
        check(self.lib.fem_solid_get_doc(self.h, d.ctypes.data_as(C.POINTER(C.c_uint8))))
        return d

    def f_e(self):
        f = np.zeros((self.N, 3))
        check(self.lib.fem_solid_force_elastic(self.h, _ptr(f)))
        return f

    def df_x(self, dx):
        dx = _f64(dx)
        df = np.zeros((self.N, 3))
        check(self.lib.fem_solid_df_x(self.h, _ptr(dx), _ptr(df)))
        return df

    def apply_A(self, factor_M, factor_K, d):
        d = _f64(d)
        q = np.zeros((self.N, 3))
        check(self.lib.fem_solid_apply_A(self.h, factor_M, factor_K, _ptr(d), _ptr(q)))
        return q

    def V(self):
        v = C.c_double()
        check(self.lib.fem_solid_energy(self.h, C.byref(v)))
        return v.value

    def mass_info(self):
        m, tv = C.c_double(), C.c_double()
        ray = np.empty(2)
        check(self.lib.fem_solid_mass_info(self.h, C.byref(m), _ptr(ray), C.byref(tv)))
        return m.value, ray, tv.value

    def stream(self):
        s = C.c_void_p()
        check(self.lib.fem_solid_stream(self.h, C.byref(s)))
        return s.value


def kernel_launches() -> int:
    return int(load().fem_kernel_launches())


def read_tetgen(node_path: str, ele_path: str, natural_scale: float = 0.0):
    """A TetGen mesh through fem_tetgen_read: (rest (N, 3) float64, tets
    (T, 4) uint32, number of tets dropped for det <= 0)."""
    lib = load()
    n, t, dropped = C.c_uint32(), C.c_uint32(), C.c_uint32()
    np_, ep = node_path.encode(), ele_path.encode()
    check(lib.fem_tetgen_read(np_, ep, natural_scale, None, 0, None, 0, C.byref(n), C.byref(t), C.byref(dropped)))
    rest = np.empty((n.value, 3))
    tets = np.empty((t.value, 4), np.uint32)
    check(lib.fem_tetgen_read(np_, ep, natural_scale, _ptr(rest), n.value, _ptr(tets, C.c_uint32), t.value,
                              C.byref(n), C.byref(t), C.byref(dropped)))
    return rest, tets, int(dropped.value)


def tetshape_rebuild(rest, tets):
    """fem_tetshape_rebuild: the tet-solid shape's rebuild of a mesh, as a
    dict of rest (V, 3), tets (T, 4), neighbors (T, 4; 0xFFFFFFFF = none),
    tet_of (T), node_of (V), bfaces (B, 3), layers (L, 2)."""
    lib = load()
    rest = _f64(rest)
    tets = np.ascontiguousarray(tets, dtype=np.uint32)
    N, T = rest.shape[0], tets.shape[0]
    out_rest = np.empty((N, 3))
    out_tets = np.empty((T, 4), np.uint32)
    nb = np.empty((T, 4), np.uint32)
    tet_of = np.empty(T, np.uint32)
    node_of = np.empty(N, np.uint32)
    bf = np.empty((4 * T, 3), np.uint32)
    layers = np.empty((T + 1, 2), np.uint32)
    V, B, L = C.c_uint32(), C.c_uint32(), C.c_uint32()
    check(lib.fem_tetshape_rebuild(_ptr(rest), N, _ptr(tets, C.c_uint32), T, _ptr(out_rest), C.byref(V),
                                   _ptr(out_tets, C.c_uint32), _ptr(nb, C.c_uint32), _ptr(tet_of, C.c_uint32),
                                   _ptr(node_of, C.c_uint32), _ptr(bf, C.c_uint32), 4 * T, C.byref(B),
                                   _ptr(layers, C.c_uint32), T + 1, C.byref(L)))
    return {"rest": out_rest[:V.value], "tets": out_tets, "neighbors": nb, "tet_of": tet_of,
            "node_of": node_of[:V.value], "bfaces": bf[:B.value], "layers": layers[:L.value]}


def geo_write(path: str, rest, tets) -> None:
    """fem_geo_write: the mesh's tet-solid shape file (.geo)."""
    rest = _f64(rest)
    tets = np.ascontiguousarray(tets, dtype=np.uint32)
    check(load().fem_geo_write(path.encode(), _ptr(rest), rest.shape[0], _ptr(tets, C.c_uint32), tets.shape[0]))


def geo_read(path: str):
    """fem_geo_read: (rest (V, 3), tets (T, 4), neighbors (T, 4)) of the
    file's tet-solid shape."""
    lib = load()
    V, T = C.c_uint32(), C.c_uint32()
    check(lib.fem_geo_read(path.encode(), None, 0, None, 0, None, C.byref(V), C.byref(T)))
    rest = np.empty((V.value, 3))
    tets = np.empty((T.value, 4), np.uint32)
    nb = np.empty((T.value, 4), np.uint32)
    check(lib.fem_geo_read(path.encode(), _ptr(rest), V.value, _ptr(tets, C.c_uint32), T.value,
                           _ptr(nb, C.c_uint32), C.byref(V), C.byref(T)))
    return rest, tets, nb


def tetgen_to_geo(base_path: str, geo_path: str, natural_scale: float = 0.0) -> None:
    """fem_tetgen_to_geo: base_path.node / base_path.ele to a shape file, as
    the reference's converter does."""
    check(load().fem_tetgen_to_geo((base_path + ".node").encode(), (base_path + ".ele").encode(), natural_scale,
                                   geo_path.encode()))


def profile_enable(on: bool = True) -> None:
    load().fem_profile_enable(1 if on else 0)


def profile_read(kernel: str):
    ms = C.c_double()
    n = C.c_ulonglong()
    load().fem_profile_read(kernel.encode(), C.byref(ms), C.byref(n))
    return ms.value, n.value


def bounds_check_status():
    """Reads and clears the kernels' index-check counts: {"enabled",
    "failures", "site", "index", "limit"} (enabled is False in the normal
    library, whose counts are always 0)."""
    en = C.c_int()
    w = [C.c_uint32() for _ in range(4)]
    check(load().fem_bounds_check_status(C.byref(en), *[C.byref(v) for v in w]))
    return {"enabled": bool(en.value), "failures": w[0].value, "site": w[1].value, "index": w[2].value,
            "limit": w[3].value}


def device_info():
    vals = [C.c_int() for _ in range(4)]
    check(load().fem_device_info(*[C.byref(v) for v in vals]))
    return {"device": vals[0].value, "sm_count": vals[1].value, "cc": (vals[2].value, vals[3].value)}


# ---------------------------------------------------------------- batches
class FemBatchOptions(C.Structure):
    _fields_ = [("precision", C.c_uint32), ("tile_elems", C.c_uint32), ("reorder", C.c_uint32),
                ("use_graph", C.c_uint32), ("chunk_nodes", C.c_uint32), ("fuse_alpha", C.c_uint32),
                ("persistent_loop", C.c_uint32)]


_u8p = C.POINTER(C.c_uint8)


def _bind_batch_signatures():
    SIGNATURES.update(_BATCH_SIGNATURES)
    SIGNATURES.update(_SERVER_SIGNATURES)


class FemServerOptions(C.Structure):
    _fields_ = [("precision", C.c_uint32), ("shard_max_scenes", C.c_uint32), ("shard_max_tets", C.c_uint64),
                ("hbm_budget_bytes", C.c_uint64), ("slice_iterations", C.c_uint32), ("chunk_nodes", C.c_uint32),
                ("fuse_alpha", C.c_uint32), ("persistent_loop", C.c_uint32)]


class FemServerCompletion(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("scene", C.c_uint32), ("status", C.c_uint32), ("cg_iterations", C.c_uint32),
                ("fp64_resolved", C.c_uint32), ("latency_us", C.c_double), ("queue_us", C.c_double),
                ("device_us", C.c_double)]


class FemServerStatus(C.Structure):
    _fields_ = [("resident_scenes", C.c_uint32), ("waiting_scenes", C.c_uint32), ("shards", C.c_uint32),
                ("busy_shards", C.c_uint32), ("max_busy_shards", C.c_uint32), ("pad", C.c_uint32),
                ("device_bytes", C.c_uint64), ("pending_requests", C.c_uint64)]


_SERVER_SIGNATURES = {
    "fem_server_options_default": (C.c_int, [C.POINTER(FemServerOptions)]),
    "fem_server_create": (C.c_int, [C.POINTER(FemServerOptions), C.POINTER(C.c_void_p)]),
    "fem_server_destroy": (C.c_int, [C.c_void_p]),
    "fem_server_add_scene": (C.c_int, [C.c_void_p, _dp, C.c_uint32, _up, C.c_uint32, C.POINTER(FemParams), _dp,
                                       _dp, _up, _dp, C.c_uint32, _up]),
    "fem_server_admit": (C.c_int, [C.c_void_p, _up]),
    "fem_server_remove_scene": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fem_server_submit": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64]),
    "fem_server_pump": (C.c_int, [C.c_void_p, C.POINTER(FemServerCompletion), C.c_uint32, _up]),
    "fem_server_get_state": (C.c_int, [C.c_void_p, C.c_uint32, _dp, _dp]),
    "fem_server_set_state": (C.c_int, [C.c_void_p, C.c_uint32, _dp, _dp]),
    "fem_server_get_status": (C.c_int, [C.c_void_p, C.POINTER(FemServerStatus)]),
    "fem_server_scene_info": (C.c_int, [C.c_void_p, C.c_uint32, _up, _up, _up]),
}


_BATCH_SIGNATURES = {
    "fem_batch_options_default": (C.c_int, [C.POINTER(FemBatchOptions)]),
    "fem_batch_create": (C.c_int, [C.POINTER(FemBatchOptions), C.POINTER(C.c_void_p)]),
    "fem_batch_add_mesh": (C.c_int, [C.c_void_p, _dp, C.c_uint32, _up, C.c_uint32, C.POINTER(FemParams), _dp, _dp,
                                     _up]),
    "fem_batch_set_knc": (C.c_int, [C.c_void_p, C.c_uint32, _up, _dp, C.c_uint32]),
    "fem_batch_finalize": (C.c_int, [C.c_void_p]),
    "fem_batch_destroy": (C.c_int, [C.c_void_p]),
    "fem_batch_info": (C.c_int, [C.c_void_p, _up, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), _up,
                                 C.POINTER(C.c_uint64)]),
    "fem_batch_set_knc_targets": (C.c_int, [C.c_void_p, C.c_uint32, _dp]),
    "fem_batch_set_state": (C.c_int, [C.c_void_p, C.c_uint32, _dp, _dp]),
    "fem_batch_get_state": (C.c_int, [C.c_void_p, C.c_uint32, _dp, _dp]),
    "fem_batch_get_rotations": (C.c_int, [C.c_void_p, C.c_uint32, _dp, _dp]),
    "fem_batch_get_dapd_state": (C.c_int, [C.c_void_p, C.c_uint32, _dp, C.POINTER(C.c_uint8)]),
    "fem_batch_set_dapd_state": (C.c_int, [C.c_void_p, C.c_uint32, _dp, C.POINTER(C.c_uint8)]),
    "fem_batch_set_active": (C.c_int, [C.c_void_p, _u8p]),
    "fem_batch_step_async": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fem_batch_synchronize": (C.c_int, [C.c_void_p]),
    "fem_batch_step": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fem_batch_get_stats": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(FemStepStats)]),
    "fem_batch_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "fem_batch_kernel_launches": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64)]),
    "fem_batch_reset_launch_count": (C.c_int, [C.c_void_p]),
    "fem_batch_set_state_all": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fem_batch_use_graph": (C.c_int, [C.c_void_p, C.c_int]),
    "fem_batch_get_state_all": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fem_batch_step_host": (C.c_int, [C.c_void_p, _dp, _dp, C.c_uint32, _dp, _dp]),
    "fem_batch_set_slice": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fem_batch_set_params": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "fem_batch_get_params": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "fem_server_set_params": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "fem_batch_nr_init": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_batch_nr_prestep": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_batch_nr_midstep": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_batch_nr_poststep": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_batch_nr_end": (C.c_int, [C.c_void_p, C.c_double]),
    "fem_batch_multi_step": (C.c_int, [C.c_void_p, C.c_double, C.c_uint32]),
    "fem_batch_set_wait_limit": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fem_batch_finished": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8)]),
}


def batch_options(precision=FEM_PRECISION_MIXED, tile_elems=256, reorder=True, use_graph=True, chunk_nodes=None,
                  fuse_alpha=False, persistent_loop=False):
    o = FemBatchOptions()
    check(load().fem_batch_options_default(C.byref(o)))
    o.precision = precision
    o.tile_elems = tile_elems
    o.reorder = 1 if reorder else 0
    o.use_graph = 1 if use_graph else 0
    if chunk_nodes is not None:
        o.chunk_nodes = chunk_nodes
    o.fuse_alpha = 1 if fuse_alpha else 0
    o.persistent_loop = 1 if persistent_loop else 0
    return o


def multi_step(solids, dt, nsteps=1):
    """fem_multi_step over Solid objects (the aggregate's lock-step); the
    schedules of driven constraints advance per step as in Solid.step."""
    lib = load()
    arr = (C.c_void_p * len(solids))(*[s.h.value if isinstance(s.h, C.c_void_p) else s.h for s in solids])
    for _ in range(nsteps):
        for s in solids:
            sc = s.scene
            if sc.knc_schedule is not None and s._knc_nodes.size:
                s.set_knc_targets(sc.targets_at(s.step_index))
            s.step_index += 1
        check(lib.fem_multi_step(arr, len(solids), float(dt), 1))


class Batch:
    """Many independent solids stepped together on one GPU (fem_batch_*)."""

    def __init__(self, scenes_list, precision=FEM_PRECISION_MIXED, tile_elems=256, reorder=True, use_graph=True,
                 chunk_nodes=None,
                 compute_energy=True, refresh_every=None, degenerate_det_F=None, rotation_check=None,
                 refresh_drop=None, rotation_fp32=None, fuse_alpha=False, persistent_loop=False):
        lib = load()
        self.lib = lib
        self.scenes = list(scenes_list)
        self.precision = precision
        h = C.c_void_p()
        opt = batch_options(precision, tile_elems, reorder, use_graph, chunk_nodes, fuse_alpha, persistent_loop)
        check(lib.fem_batch_create(C.byref(opt), C.byref(h)))
        self.h = h
        self._knc = []
        for sc in self.scenes:
            p = params_for(sc, precision, compute_energy)
            if refresh_every is not None:
                p.refresh_every = refresh_every
            if degenerate_det_F is not None:
                p.degenerate_det_F = degenerate_det_F
            if rotation_check is not None:
                p.rotation_check = rotation_check
            if refresh_drop is not None:
                p.refresh_drop = refresh_drop
            if rotation_fp32 is not None:
                p.rotation_fp32 = rotation_fp32
            rest = _f64(sc.rest)
            tets = np.ascontiguousarray(sc.tets, dtype=np.uint32)
            idx = C.c_uint32()
            check(lib.fem_batch_add_mesh(h, _ptr(rest), sc.num_nodes, _ptr(tets, C.c_uint32), sc.num_tets,
                                         C.byref(p), _ptr(_f64(sc.young_per_elem)), _ptr(_f64(sc.poisson_per_elem)),
                                         C.byref(idx)))
            nodes = np.ascontiguousarray(sc.knc_nodes, dtype=np.uint32)
            self._knc.append(nodes)
            if nodes.size:
                tg = _f64(sc.targets_at(0) if sc.knc_schedule is not None else sc.knc_targets)
                check(lib.fem_batch_set_knc(h, idx.value, _ptr(nodes, C.c_uint32), _ptr(tg), nodes.size))
        check(lib.fem_batch_finalize(h))
        for i, sc in enumerate(self.scenes):
            if sc.init_vel is not None:
                self.set_state(i, v=sc.init_vel)
        self.step_index = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.fem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_slice(self, max_iterations):
        check(self.lib.fem_batch_set_slice(self.h, int(max_iterations)))

    def set_wait_limit(self, polls=None):
        """Poll limit of the tile product's waits for a tile copy (None: the
        default, 2^22)."""
        check(self.lib.fem_batch_set_wait_limit(self.h, FEM_WAIT_LIMIT_DEFAULT if polls is None else int(polls)))

    def finished(self):
        f = np.zeros(len(self.scenes), np.uint8)
        check(self.lib.fem_batch_finished(self.h, f.ctypes.data_as(C.POINTER(C.c_uint8))))
        return f

    def info(self):
        m, t = C.c_uint32(), C.c_uint32()
        n, e, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(self.lib.fem_batch_info(self.h, C.byref(m), C.byref(n), C.byref(e), C.byref(t), C.byref(b)))
        return {"meshes": m.value, "nodes": n.value, "tets": e.value, "tiles": t.value, "device_bytes": b.value}

    def set_state(self, i, x=None, v=None):
        x, v = _f64(x), _f64(v)
        check(self.lib.fem_batch_set_state(self.h, i, _ptr(x), _ptr(v)))

    def state(self, i):
        n = self.scenes[i].num_nodes
        x = np.empty((n, 3))
        v = np.empty((n, 3))
        check(self.lib.fem_batch_get_state(self.h, i, _ptr(x), _ptr(v)))
        return x, v

    def rotations(self, i):
        """Rotations (T, 3, 3) and det F (T) of mesh i as of its last
        BeginEvaluation, in the caller's element order."""
        t = self.scenes[i].num_tets
        R = np.empty((t, 3, 3))
        d = np.empty(t)
        check(self.lib.fem_batch_get_rotations(self.h, i, _ptr(R), _ptr(d)))
        return R, d

    def dapd_state(self, i):
        """DAPD mesh i's previous positions (N, 3) and directions of collapse (T, 2)."""
        sc = self.scenes[i]
        px = np.empty((sc.num_nodes, 3))
        doc = np.empty((sc.num_tets, 2), np.uint8)
        check(self.lib.fem_batch_get_dapd_state(self.h, i, _ptr(px), doc.ctypes.data_as(C.POINTER(C.c_uint8))))
        return px, doc

    def set_dapd_state(self, i, prev_x=None, doc=None):
        px = _f64(prev_x)
        d = None if doc is None else np.ascontiguousarray(doc, dtype=np.uint8)
        check(self.lib.fem_batch_set_dapd_state(self.h, i, _ptr(px),
                                                None if d is None else d.ctypes.data_as(C.POINTER(C.c_uint8))))

    def set_active(self, mask=None):
        if mask is None:
            check(self.lib.fem_batch_set_active(self.h, None))
        else:
            m = np.ascontiguousarray(mask, dtype=np.uint8)
            check(self.lib.fem_batch_set_active(self.h, m.ctypes.data_as(_u8p)))

    def _drive_targets(self):
        for i, sc in enumerate(self.scenes):
            if sc.knc_schedule is not None and self._knc[i].size:
                tg = _f64(sc.targets_at(self.step_index))
                check(self.lib.fem_batch_set_knc_targets(self.h, i, _ptr(tg)))

    def step(self, n=1):
        for _ in range(n):
            self._drive_targets()
            check(self.lib.fem_batch_step_async(self.h, 1))
            self.step_index += 1
        check(self.lib.fem_batch_synchronize(self.h))

    def stats(self, i):
        st = FemStepStats()
        check(self.lib.fem_batch_get_stats(self.h, i, C.byref(st)))
        return st.as_dict()

    def set_params(self, i, params):
        """fem_batch_set_params: mesh i takes new parameters (a FemParams,
        e.g. params_for(scene)) between steps."""
        check(self.lib.fem_batch_set_params(self.h, i, C.byref(params)))

    def get_params(self, i):
        p = FemParams()
        check(self.lib.fem_batch_get_params(self.h, i, C.byref(p)))
        return p

    def nr_phase(self, phase, dt):
        """One lock-step phase (init, prestep, midstep, poststep, end;
        fem_batch_nr_*) on every solid taking part; init advances the
        schedules of driven constraints as a step does."""
        if phase == "init":
            self._drive_targets()
            self.step_index += 1
        check(getattr(self.lib, "fem_batch_nr_" + phase)(self.h, float(dt)))

    def multi_step(self, dt, nsteps=1):
        """fem_batch_multi_step: the aggregate's lock-step over the batch's
        solids, one step per call so that driven constraints advance."""
        for _ in range(nsteps):
            self._drive_targets()
            check(self.lib.fem_batch_multi_step(self.h, float(dt), 1))
            self.step_index += 1

    def stream(self):
        s = C.c_void_p()
        check(self.lib.fem_batch_stream(self.h, C.byref(s)))
        return s.value

    def kernel_launches(self, steps):
        n = C.c_uint64()
        check(self.lib.fem_batch_kernel_launches(self.h, steps, C.byref(n)))
        return n.value

    def reset_launch_count(self):
        check(self.lib.fem_batch_reset_launch_count(self.h))


class Server:
    """Step requests over device-resident scenes (fem_server_*): admission by
    a device-memory budget, size-sorted shards, continuous batching."""

    def __init__(self, precision=FEM_PRECISION_MIXED, hbm_budget_bytes=None, shard_max_tets=None,
                 shard_max_scenes=None, slice_iterations=None, completion_capacity=65536, chunk_nodes=None,
                 fuse_alpha=None, persistent_loop=None):
        lib = load()
        self.lib = lib
        opt = FemServerOptions()
        check(lib.fem_server_options_default(C.byref(opt)))
        opt.precision = precision
        if hbm_budget_bytes is not None:
            opt.hbm_budget_bytes = int(hbm_budget_bytes)
        if shard_max_tets is not None:
            opt.shard_max_tets = int(shard_max_tets)
        if shard_max_scenes is not None:
            opt.shard_max_scenes = int(shard_max_scenes)
        if slice_iterations is not None:
            opt.slice_iterations = int(slice_iterations)
        if chunk_nodes is not None:
            opt.chunk_nodes = int(chunk_nodes)
        if fuse_alpha is not None:
            opt.fuse_alpha = 1 if fuse_alpha else 0
        if persistent_loop is not None:
            opt.persistent_loop = 1 if persistent_loop else 0
        h = C.c_void_p()
        check(lib.fem_server_create(C.byref(opt), C.byref(h)))
        self.h = h
        self.precision = precision
        self.scenes = []
        self._cap = completion_capacity
        self._buf = (FemServerCompletion * completion_capacity)()

    def close(self):
        if getattr(self, "h", None):
            self.lib.fem_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, sc, compute_energy=False):
        p = params_for(sc, self.precision, compute_energy)
        rest = _f64(sc.rest)
        tets = np.ascontiguousarray(sc.tets, dtype=np.uint32)
        nodes = np.ascontiguousarray(sc.knc_nodes, dtype=np.uint32)
        tg = _f64(sc.knc_targets) if nodes.size else None
        idx = C.c_uint32()
        check(self.lib.fem_server_add_scene(self.h, _ptr(rest), sc.num_nodes, _ptr(tets, C.c_uint32), sc.num_tets,
                                            C.byref(p), _ptr(_f64(sc.young_per_elem)),
                                            _ptr(_f64(sc.poisson_per_elem)),
                                            _ptr(nodes, C.c_uint32) if nodes.size else None,
                                            _ptr(tg) if nodes.size else None, int(nodes.size), C.byref(idx)))
        self.scenes.append(sc)
        return idx.value

    def admit(self):
        n = C.c_uint32()
        check(self.lib.fem_server_admit(self.h, C.byref(n)))
        return n.value

    def set_params(self, scene, params):
        """fem_server_set_params: run-time parameter change of a scene with
        no request pending."""
        check(self.lib.fem_server_set_params(self.h, scene, C.byref(params)))

    def remove(self, scene):
        check(self.lib.fem_server_remove_scene(self.h, scene))

    def submit(self, scene, tag=0):
        check(self.lib.fem_server_submit(self.h, scene, tag))

    def pump(self):
        """Completions of this call as a list of dicts."""
        n = C.c_uint32()
        check(self.lib.fem_server_pump(self.h, self._buf, self._cap, C.byref(n)))
        out = []
        for i in range(n.value):
            c = self._buf[i]
            out.append({"tag": c.tag, "scene": c.scene, "status": c.status, "cg_iterations": c.cg_iterations,
                        "fp64_resolved": c.fp64_resolved, "latency_us": c.latency_us, "queue_us": c.queue_us,
                        "device_us": c.device_us})
        return out

    def drain(self, timeout_s=600.0):
        """Pump until no request is pending."""
        import time
        done, t0 = [], time.perf_counter()
        while self.status()["pending_requests"]:
            done += self.pump()
            if time.perf_counter() - t0 > timeout_s:
                raise FemError(FEM_E_TIMEOUT, "server drain timed out")
        return done

    def state(self, scene):
        n = self.scenes[scene].num_nodes
        x = np.empty((n, 3))
        v = np.empty((n, 3))
        check(self.lib.fem_server_get_state(self.h, scene, _ptr(x), _ptr(v)))
        return x, v

    def set_state(self, scene, x=None, v=None):
        x, v = _f64(x), _f64(v)
        check(self.lib.fem_server_set_state(self.h, scene, _ptr(x), _ptr(v)))

    def scene_info(self, scene):
        state, shard, pending = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(self.lib.fem_server_scene_info(self.h, scene, C.byref(state), C.byref(shard), C.byref(pending)))
        return {"state": ("waiting", "resident", "removed")[state.value], "shard": shard.value,
                "pending": pending.value}

    def resident(self):
        return [i for i in range(len(self.scenes)) if self.scene_info(i)["state"] == "resident"]

    def status(self):
        st = FemServerStatus()
        check(self.lib.fem_server_get_status(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in FemServerStatus._fields_ if k != "pad"}

