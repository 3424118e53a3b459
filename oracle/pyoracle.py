"""TEST INFRASTRUCTURE ONLY -- ctypes access to the oracle libraries.

Two libraries with the same solid interface:
  * ``port``: the plain-C restatement (oracle/_build/libfemoracle.so);
  * ``ref_dbl``: the reference's own FP64 translation units plus the
    restated Leaf driver, with Mal's Sqrt/Sin/Cos/ATan2 evaluated at double
    precision (oracle/_ref/libfemref_dbl.so) -- the build the restatement is
    pinned to;
  * ``ref``: the same translation units as written (oracle/_ref/libfemref.so),
    whose float-rounded Sqrt makes rotations NaN near F = I.
The reference builds exist only where the reference sources were present at
build time and are limited to 65535 nodes/elements (uint16 indices).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libfemoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfemref.so")
REF_DBL_SO = os.path.join(HERE, "_ref", "libfemref_dbl.so")
GEO_REF_SO = os.path.join(HERE, "_ref", "libgeoref.so")
# The reference tree (read only to build the checker): REFERENCE_ROOT from
# the environment, the same variable oracle/Makefile reads.
REFERENCE_ROOT = os.environ.get("REFERENCE_ROOT", "/root/reference")
REFERENCE_SRC = os.path.join(REFERENCE_ROOT, "src")

MATH_DOUBLE = 0
MATH_FLOAT_LITERAL = 1

_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)


def build(reference: bool = False) -> None:
    """Compile the restatement (and the reference checker when its sources
    are present and `reference` is true)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if reference and os.path.isdir(REFERENCE_SRC):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_ROOT}"])


def geo_ref_convert(pos, tets, natural_scale, out_path):
    """The reference's TetGen converter path on (float positions, tets as
    read from the files): its EditableTetSolidShape3 and shape library
    (oracle/geo_harness.cpp) write out_path. Returns the harness status."""
    lib = C.CDLL(GEO_REF_SO)
    lib.geo_ref_convert.argtypes = [C.POINTER(C.c_float), C.c_uint32, _up, C.c_uint32, C.c_float, C.c_char_p]
    lib.geo_ref_convert.restype = C.c_int
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    tets = np.ascontiguousarray(tets, dtype=np.uint32)
    return lib.geo_ref_convert(pos.ctypes.data_as(C.POINTER(C.c_float)), pos.shape[0], _ptr(tets, C.c_uint32),
                               tets.shape[0], natural_scale, out_path.encode())


def _ptr(a, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


_LIBS = {}


def _load(path: str, prefix: str):
    key = (path, prefix)
    if key in _LIBS:
        return _LIBS[key]
    lib = C.CDLL(path)
    P = prefix
    fn = lambda n: getattr(lib, P + n)
    args_create = [C.c_uint32, _dp, C.c_uint32, _up, C.c_double, C.c_double, _dp, _dp,
                   C.c_double, C.c_double, _dp, C.c_double, C.c_double, C.c_double, C.c_uint32]
    if P == "orc_":
        args_create = args_create + [C.c_int]
    fn("solid_create").argtypes = args_create
    fn("solid_create").restype = C.c_void_p
    fn("solid_destroy").argtypes = [C.c_void_p]
    fn("solid_set_knc").argtypes = [C.c_void_p, C.c_uint32, _up, _dp]
    fn("solid_set_knc_targets").argtypes = [C.c_void_p, _dp]
    fn("solid_set_state").argtypes = [C.c_void_p, _dp, _dp]
    fn("solid_get_state").argtypes = [C.c_void_p, _dp, _dp]
    fn("solid_fixed_step").argtypes = [C.c_void_p]
    fn("solid_last_stats").argtypes = [C.c_void_p, _up, _dp, _dp, _dp, _dp]
    fn("solid_rayleigh").argtypes = [C.c_void_p, _dp]
    fn("solid_node_mass").argtypes = [C.c_void_p]
    fn("solid_node_mass").restype = C.c_double
    fn("solid_set_integrator").argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double]
    fn("solid_set_rotation").argtypes = [C.c_void_p, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_double]
    fn("solid_set_ls_solver").argtypes = [C.c_void_p, C.c_uint32]
    fn("solid_set_material").argtypes = [C.c_void_p, C.c_uint32]
    fn("solid_set_ecie_k_factor").argtypes = [C.c_void_p, C.c_double]
    fn("solid_last_nr_stats").argtypes = [C.c_void_p, _up, _dp, _dp]
    for ph in ("init", "prestep", "midstep", "poststep", "end"):
        fn("solid_nr_" + ph).argtypes = [C.c_void_p, C.c_double]
    fn("multi_lock_step").argtypes = [C.POINTER(C.c_void_p), C.c_uint32, C.c_double]
    fn("solid_last_lock_stats").argtypes = [C.c_void_p, _up, _up]
    if P == "orc_":
        lib.orc_solid_begin_eval.argtypes = [C.c_void_p, _dp]
        lib.orc_solid_rotations.argtypes = [C.c_void_p, _dp]
        lib.orc_solid_detF.argtypes = [C.c_void_p, _dp]
        lib.orc_solid_f_e.argtypes = [C.c_void_p, _dp]
        lib.orc_solid_df_x.argtypes = [C.c_void_p, _dp, _dp]
        lib.orc_solid_V.argtypes = [C.c_void_p]
        lib.orc_solid_V.restype = C.c_double
        lib.orc_solid_apply_A.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp, _dp]
        lib.orc_rotation_svd.argtypes = [_dp, _dp, C.c_int]
        lib.orc_solid_element_K.argtypes = [C.c_void_p, C.c_uint32, _dp]
        lib.orc_solid_set_solver.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_uint32]
        lib.orc_solid_doc.argtypes = [C.c_void_p, C.POINTER(C.c_uint8)]
        lib.orc_solid_set_threads.argtypes = [C.c_void_p, C.c_int]
        lib.orc_solid_total_volume.argtypes = [C.c_void_p]
        lib.orc_solid_total_volume.restype = C.c_double
    else:
        lib.ref_real_size.restype = C.c_int
        lib.ref_rotation_svd.argtypes = [_dp, _dp]
        lib.ref_tes_create.argtypes = [C.c_uint32, _dp, C.c_uint32, _up, C.c_double, C.c_double, _dp, _dp]
        lib.ref_tes_create.restype = C.c_void_p
        lib.ref_tes_destroy.argtypes = [C.c_void_p]
        lib.ref_tes_begin_eval.argtypes = [C.c_void_p, _dp]
        lib.ref_tes_rotations.argtypes = [C.c_void_p, _dp]
        lib.ref_tes_f_e.argtypes = [C.c_void_p, _dp]
        lib.ref_tes_df_x.argtypes = [C.c_void_p, _dp, _dp]
        lib.ref_tes_V.argtypes = [C.c_void_p]
        lib.ref_tes_V.restype = C.c_double
    _LIBS[key] = lib
    return lib


class Solid:
    """One solid stepped by the oracle restatement (kind='port', with
    math=MATH_DOUBLE or MATH_FLOAT_LITERAL) or a reference build
    (kind='ref_dbl' or 'ref')."""

    def __init__(self, scene, kind: str = "port", math: int = MATH_DOUBLE):
        self.kind = kind
        if kind == "port":
            self.lib = _load(PORT_SO, "orc_")
            self.p = "orc_"
        else:
            self.lib = _load(REF_DBL_SO if kind == "ref_dbl" else REF_SO, "ref_")
            self.p = "ref_"
        self.scene = scene
        self.N = scene.num_nodes
        self.T = scene.num_tets
        self._rest = _f64(scene.rest)
        self._tets = np.ascontiguousarray(scene.tets, dtype=np.uint32)
        self._Ep = _f64(scene.young_per_elem)
        self._nup = _f64(scene.poisson_per_elem)
        self._g = np.asarray(scene.gravity, dtype=np.float64)
        args = [self.N, _ptr(self._rest), self.T, _ptr(self._tets, C.c_uint32), scene.young, scene.poisson,
                _ptr(self._Ep), _ptr(self._nup), scene.density, scene.damping_ratio, _ptr(self._g),
                scene.dt, scene.rel_eps, scene.abs_eps, scene.max_iter]
        if kind == "port":
            args.append(math)
        self.h = getattr(self.lib, self.p + "solid_create")(*args)
        if not self.h:
            raise ValueError("oracle solid_create rejected the scene")
        nodes = np.ascontiguousarray(scene.knc_nodes, dtype=np.uint32)
        self._knc_nodes = nodes
        if nodes.size:
            tg = _f64(scene.targets_at(0) if scene.knc_schedule is not None else scene.knc_targets)
            getattr(self.lib, self.p + "solid_set_knc")(self.h, nodes.size, _ptr(nodes, C.c_uint32), _ptr(tg))
        if scene.init_vel is not None:
            v = _f64(scene.init_vel)
            getattr(self.lib, self.p + "solid_set_state")(self.h, None, _ptr(v))
        if getattr(scene, "rotation", 0):
            getattr(self.lib, self.p + "solid_set_rotation")(self.h, scene.rotation, scene.dapd_threshold,
                                                              scene.dapd_L, scene.dapd_NL, scene.dapd_exponent)
        if getattr(scene, "material", 0):
            getattr(self.lib, self.p + "solid_set_material")(self.h, scene.material)
        if getattr(scene, "ecie_k_factor", 1.0) != 1.0:
            getattr(self.lib, self.p + "solid_set_ecie_k_factor")(self.h, scene.ecie_k_factor)
        if getattr(scene, "ls_solver", 0):
            getattr(self.lib, self.p + "solid_set_ls_solver")(self.h, scene.ls_solver)
        if getattr(scene, "integrator", 0):
            getattr(self.lib, self.p + "solid_set_integrator")(self.h, scene.integrator, scene.nr_max_iter,
                                                                scene.nr_abs_eps)
        self.step_index = 0

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            getattr(self.lib, self.p + "solid_destroy")(h)
            self.h = None

    def set_state(self, x=None, v=None):
        x = _f64(x)
        v = _f64(v)
        getattr(self.lib, self.p + "solid_set_state")(self.h, _ptr(x), _ptr(v))

    def state(self):
        x = np.empty((self.N, 3))
        v = np.empty((self.N, 3))
        getattr(self.lib, self.p + "solid_get_state")(self.h, _ptr(x), _ptr(v))
        return x, v

    def step(self):
        sc = self.scene
        if sc.knc_schedule is not None and self._knc_nodes.size:
            tg = _f64(sc.targets_at(self.step_index))
            getattr(self.lib, self.p + "solid_set_knc_targets")(self.h, _ptr(tg))
        getattr(self.lib, self.p + "solid_fixed_step")(self.h)
        self.step_index += 1
        return self.last_stats()

    def last_stats(self):
        it = C.c_uint32()
        rel, ab, ee, pe = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        getattr(self.lib, self.p + "solid_last_stats")(self.h, C.byref(it), C.byref(rel), C.byref(ab),
                                                        C.byref(ee), C.byref(pe))
        nr_it = C.c_uint32()
        nr_rel, nr_abs = C.c_double(), C.c_double()
        getattr(self.lib, self.p + "solid_last_nr_stats")(self.h, C.byref(nr_it), C.byref(nr_rel), C.byref(nr_abs))
        return {"iters": it.value, "rel_res": rel.value, "abs_res": ab.value,
                "elastic_energy": ee.value, "potential_energy": pe.value,
                "nr_iters": nr_it.value, "nr_rel": nr_rel.value, "nr_abs": nr_abs.value}

    def run(self, steps=None):
        steps = self.scene.steps if steps is None else steps
        stats = [self.step() for _ in range(steps)]
        return stats

    def node_mass(self):
        return getattr(self.lib, self.p + "solid_node_mass")(self.h)

    def rayleigh(self):
        out = np.empty(2)
        getattr(self.lib, self.p + "solid_rayleigh")(self.h, _ptr(out))
        return out

    def set_knc_targets_at(self, step: int):
        """Targets of the driven constraints at `step` of the scene's schedule."""
        tg = _f64(self.scene.targets_at(step))
        getattr(self.lib, self.p + "solid_set_knc_targets")(self.h, _ptr(tg))

    def nr_phase(self, phase: str, dt: float):
        """One multi-solid Newton lock-step phase: init, prestep, midstep,
        poststep or end (the Leaf's NR_* methods)."""
        getattr(self.lib, self.p + "solid_nr_" + phase)(self.h, dt)

    def lock_stats(self):
        k, ls = C.c_uint32(), C.c_uint32()
        getattr(self.lib, self.p + "solid_last_lock_stats")(self.h, C.byref(k), C.byref(ls))
        return {"nr_iters": k.value, "iters": ls.value}

    def set_threads(self, threads: int):
        """Host threads of the element loops (port only); results are
        bit-identical for any count."""
        self.lib.orc_solid_set_threads(self.h, int(threads))
        return self

    def set_solver(self, rel_eps, abs_eps, max_iter):
        self.lib.orc_solid_set_solver(self.h, rel_eps, abs_eps, max_iter)

    def reset(self):
        """Back to the scene's initial state (positions at rest, initial velocity)."""
        v0 = np.zeros_like(self._rest) if self.scene.init_vel is None else self.scene.init_vel
        self.set_state(self._rest, v0)
        self.step_index = 0

    # ---- element-level hooks (port only) ----
    def begin_eval(self, x):
        x = _f64(x)
        self.lib.orc_solid_begin_eval(self.h, _ptr(x))

    def rotations(self):
        R = np.empty((self.T, 3, 3))
        self.lib.orc_solid_rotations(self.h, _ptr(R))
        return R

    def detF(self):
        d = np.empty(self.T)
        self.lib.orc_solid_detF(self.h, _ptr(d))
        return d

    def f_e(self):
        f = np.zeros((self.N, 3))
        self.lib.orc_solid_f_e(self.h, _ptr(f))
        return f

    def df_x(self, dx):
        dx = _f64(dx)
        df = np.zeros((self.N, 3))
        self.lib.orc_solid_df_x(self.h, _ptr(dx), _ptr(df))
        return df

    def apply_A(self, factor_M, factor_K, d):
        d = _f64(d)
        q = np.zeros((self.N, 3))
        self.lib.orc_solid_apply_A(self.h, factor_M, factor_K, _ptr(d), _ptr(q))
        return q

    def V(self):
        return self.lib.orc_solid_V(self.h)

    def doc(self):
        """Per-element direction of collapse (vit0, vit1); (3, 0) = none."""
        d = np.empty((self.T, 2), np.uint8)
        self.lib.orc_solid_doc(self.h, d.ctypes.data_as(C.POINTER(C.c_uint8)))
        return d

    def element_K(self, e):
        K = np.empty((4, 4, 3, 3))
        self.lib.orc_solid_element_K(self.h, e, _ptr(K))
        return K


def multi_lock_step(solids, dt: float):
    """One fixed step of the multi-solid aggregate
    (SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update, contacts off) over
    oracle solids of one kind; the schedules of driven constraints advance
    as in Solid.step."""
    lib, p = solids[0].lib, solids[0].p
    for s in solids:
        sc = s.scene
        if sc.knc_schedule is not None and s._knc_nodes.size:
            tg = _f64(sc.targets_at(s.step_index))
            getattr(lib, p + "solid_set_knc_targets")(s.h, _ptr(tg))
        s.step_index += 1
    arr = (C.c_void_p * len(solids))(*[s.h for s in solids])
    getattr(lib, p + "multi_lock_step")(arr, len(solids), dt)


class RefElementSet:
    """The reference's TetrahedronElementSet3 alone (element-level parity)."""

    def __init__(self, scene, dbl: bool = True):
        self.lib = _load(REF_DBL_SO if dbl else REF_SO, "ref_")
        self.N, self.T = scene.num_nodes, scene.num_tets
        self._rest = _f64(scene.rest)
        self._tets = np.ascontiguousarray(scene.tets, dtype=np.uint32)
        self._Ep = _f64(scene.young_per_elem)
        self._nup = _f64(scene.poisson_per_elem)
        self.h = self.lib.ref_tes_create(self.N, _ptr(self._rest), self.T, _ptr(self._tets, C.c_uint32),
                                         scene.young, scene.poisson, _ptr(self._Ep), _ptr(self._nup))
        if not self.h:
            raise ValueError("reference element set rejected the mesh (uint16 index limit)")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_tes_destroy(self.h)
            self.h = None

    def begin_eval(self, x):
        x = _f64(x)
        self.lib.ref_tes_begin_eval(self.h, _ptr(x))

    def rotations(self):
        R = np.empty((self.T, 3, 3))
        self.lib.ref_tes_rotations(self.h, _ptr(R))
        return R

    def f_e(self):
        f = np.zeros((self.N, 3))
        self.lib.ref_tes_f_e(self.h, _ptr(f))
        return f

    def df_x(self, dx):
        dx = _f64(dx)
        df = np.zeros((self.N, 3))
        self.lib.ref_tes_df_x(self.h, _ptr(dx), _ptr(df))
        return df

    def V(self):
        return self.lib.ref_tes_V(self.h)


def rotation_svd(F, kind: str = "port", math: int = MATH_DOUBLE):
    F = _f64(F).reshape(3, 3)
    R = np.empty((3, 3))
    if kind == "port":
        _load(PORT_SO, "orc_").orc_rotation_svd(_ptr(F), _ptr(R), math)
    else:
        _load(REF_DBL_SO if kind == "ref_dbl" else REF_SO, "ref_").ref_rotation_svd(_ptr(F), _ptr(R))
    return R
