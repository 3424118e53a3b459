"""The C_LCM element arithmetic of the CUDA kernels (risdsdgcfem_thesis_gb300/
csrc/lcm.cuh, host-callable) against the oracle restatement, on the CPU: the
header is compiled with g++ into a small shared library and summed per node
in element order, as the oracle accumulates. F and Dm^-1 are formed here in
numpy (rounding may differ from the oracle's in the last bits), so the bar
is 1e-11 relative: it checks the formulas, not the rounding.
"""
import ctypes as C
import dataclasses
import os
import shutil
import subprocess

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = r"""
#include "lcm.cuh"
#include <stdint.h>
extern "C" {
// f[n] += force contributions (the oracle's sign), element order
void lcm_all(int mode, uint32_t T, const uint32_t* tets, const double* R, const double* F, const double* Dinv,
             const double* vol, double mu, double lam, const double* dx, double* f, double* energy)
{
    double acc = 0;
    for (uint32_t e = 0; e < T; e++) {
        const uint32_t* t = tets + 4 * e;
        double out[12];
        if (mode == 0) femgb::lcm_force(R + 9 * e, F + 9 * e, Dinv + 9 * e, vol[e], mu, lam, out);
        else if (mode == 1) {
            double dl[12];
            for (int i = 0; i < 4; i++)
                for (int a = 0; a < 3; a++) dl[3 * i + a] = dx[3 * t[i] + a];
            femgb::lcm_dforce(R + 9 * e, Dinv + 9 * e, vol[e], mu, lam, dl, out);
        } else {
            acc += femgb::lcm_energy(R + 9 * e, F + 9 * e, vol[e], mu, lam);
            continue;
        }
        for (int i = 0; i < 4; i++)
            for (int a = 0; a < 3; a++) f[3 * t[i] + a] += -out[3 * i + a];
    }
    *energy = acc;
}
// the same through the P-K dispatch (kind: 1 C_LCM, 2 C_LCMH, 3 C_CCM)
void pk_all(int kind, int mode, uint32_t T, const uint32_t* tets, const double* R, const double* F,
            const double* detF, const double* Dinv, const double* vol, double mu, double lam, double k,
            const double* dx, double* f, double* energy)
{
    femgb::PkMaterial m;
    m.kind = kind; m.mu = mu; m.lambda = lam; m.k = k;
    double acc = 0;
    for (uint32_t e = 0; e < T; e++) {
        const uint32_t* t = tets + 4 * e;
        double out[12];
        if (mode == 0) femgb::pk_force(m, R + 9 * e, F + 9 * e, Dinv + 9 * e, vol[e], out);
        else if (mode == 1) {
            double dl[12];
            for (int i = 0; i < 4; i++)
                for (int a = 0; a < 3; a++) dl[3 * i + a] = dx[3 * t[i] + a];
            femgb::pk_dforce(m, R + 9 * e, F + 9 * e, detF[e], Dinv + 9 * e, vol[e], dl, out);
        } else {
            acc += femgb::pk_energy(m, R + 9 * e, F + 9 * e, vol[e]);
            continue;
        }
        for (int i = 0; i < 4; i++)
            for (int a = 0; a < 3; a++) f[3 * t[i] + a] += -out[3 * i + a];
    }
    *energy = acc;
}
}
"""


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("lcm")
    src = d / "shim.cpp"
    src.write_text(SHIM)
    so = d / "libshim.so"
    r = subprocess.run([cxx, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                        os.path.join(ROOT, "risdsdgcfem_thesis_gb300", "csrc"), str(src), "-o", str(so)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(so))
    dp = C.POINTER(C.c_double)
    lib.lcm_all.argtypes = [C.c_int, C.c_uint32, C.POINTER(C.c_uint32), dp, dp, dp, dp, C.c_double, C.c_double,
                            dp, dp, dp]
    lib.pk_all.argtypes = [C.c_int, C.c_int, C.c_uint32, C.POINTER(C.c_uint32), dp, dp, dp, dp, dp, C.c_double,
                           C.c_double, C.c_double, dp, dp, dp]
    return lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_lcm_element_math_matches_oracle(shim, oracle):
    rng = np.random.default_rng(4)
    sc = dataclasses.replace(scenes.random_block(rng, dims=(3, 3, 2)), material=1)
    x = sc.rest + 0.02 * rng.standard_normal(sc.rest.shape) * sc.h / 0.1
    o = oracle.Solid(sc, "port")
    o.begin_eval(x)
    R = np.ascontiguousarray(o.rotations())
    tets = np.ascontiguousarray(sc.tets, np.uint32)
    Dm = np.stack([sc.rest[tets[:, j]] - sc.rest[tets[:, 0]] for j in (1, 2, 3)], axis=2)
    Ds = np.stack([x[tets[:, j]] - x[tets[:, 0]] for j in (1, 2, 3)], axis=2)
    Dinv = np.ascontiguousarray(np.linalg.inv(Dm))
    F = np.ascontiguousarray(Ds @ Dinv)
    vol = np.ascontiguousarray(np.linalg.det(Dm) / 6.0)
    E, nu = sc.young, sc.poisson
    mu, lam = 0.5 * E / (1 + nu), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    dx = np.ascontiguousarray(rng.standard_normal(sc.rest.shape))
    en = C.c_double()
    up = tets.ctypes.data_as(C.POINTER(C.c_uint32))
    f = np.zeros_like(sc.rest)
    shim.lcm_all(0, tets.shape[0], up, _p(R), _p(F), _p(Dinv), _p(vol), mu, lam, _p(dx), _p(f), C.byref(en))
    fo = o.f_e()
    assert np.linalg.norm(f - fo) <= 1e-11 * np.linalg.norm(fo)
    df = np.zeros_like(sc.rest)
    shim.lcm_all(1, tets.shape[0], up, _p(R), _p(F), _p(Dinv), _p(vol), mu, lam, _p(dx), _p(df), C.byref(en))
    dfo = o.df_x(dx)
    assert np.linalg.norm(df - dfo) <= 1e-11 * np.linalg.norm(dfo)
    shim.lcm_all(2, tets.shape[0], up, _p(R), _p(F), _p(Dinv), _p(vol), mu, lam, _p(dx), _p(df), C.byref(en))
    assert abs(en.value - o.V()) <= 1e-11 * abs(o.V())
    # and it is not the warped-stiffness force
    w = oracle.Solid(dataclasses.replace(sc, material=0), "port")
    w.begin_eval(x)
    assert np.linalg.norm(w.f_e() - fo) > 1e-6 * np.linalg.norm(fo)


@pytest.mark.parametrize("kind,k", [(2, 1.0), (2, 0.05), (3, 1.0)])
def test_lcmh_and_ccm_element_math_matches_oracle(shim, oracle, kind, k):
    """C_LCMH (blend radius k) and C_CCM: f_e, df_x and V of the header against
    the oracle at a deformed state (1e-11, numpy-formed F and Dm^-1)."""
    rng = np.random.default_rng(6)
    sc = dataclasses.replace(scenes.random_block(rng, dims=(3, 3, 2)), material=kind, ecie_k_factor=k)
    x = sc.rest + 0.02 * rng.standard_normal(sc.rest.shape) * sc.h / 0.1
    o = oracle.Solid(sc, "port")
    o.begin_eval(x)
    R = np.ascontiguousarray(o.rotations())
    detF = np.ascontiguousarray(o.detF())
    tets = np.ascontiguousarray(sc.tets, np.uint32)
    Dm = np.stack([sc.rest[tets[:, j]] - sc.rest[tets[:, 0]] for j in (1, 2, 3)], axis=2)
    Ds = np.stack([x[tets[:, j]] - x[tets[:, 0]] for j in (1, 2, 3)], axis=2)
    Dinv = np.ascontiguousarray(np.linalg.inv(Dm))
    F = np.ascontiguousarray(Ds @ Dinv)
    vol = np.ascontiguousarray(np.linalg.det(Dm) / 6.0)
    E, nu = sc.young, sc.poisson
    mu, lam = 0.5 * E / (1 + nu), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    dx = np.ascontiguousarray(rng.standard_normal(sc.rest.shape))
    en = C.c_double()
    up = tets.ctypes.data_as(C.POINTER(C.c_uint32))
    args = (tets.shape[0], up, _p(R), _p(F), _p(detF), _p(Dinv), _p(vol), mu, lam, float(np.float32(k)), _p(dx))
    f = np.zeros_like(sc.rest)
    shim.pk_all(kind, 0, *args, _p(f), C.byref(en))
    fo = o.f_e()
    assert np.linalg.norm(f - fo) <= 1e-11 * np.linalg.norm(fo)
    df = np.zeros_like(sc.rest)
    shim.pk_all(kind, 1, *args, _p(df), C.byref(en))
    dfo = o.df_x(dx)
    assert np.linalg.norm(df - dfo) <= 1e-11 * np.linalg.norm(dfo)
    shim.pk_all(kind, 2, *args, _p(df), C.byref(en))
    assert abs(en.value - o.V()) <= 1e-11 * max(abs(o.V()), 1e-300)
