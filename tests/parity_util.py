"""Shared helpers for the GPU parity tests."""
import copy

import numpy as np


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def perturbed(sc, seed, eps=1e-15):
    p = copy.copy(sc)
    v0 = np.zeros_like(sc.rest) if sc.init_vel is None else sc.init_vel
    p.init_vel = v0 + eps * np.abs(sc.rest).max() * np.random.default_rng(seed).standard_normal(sc.rest.shape)
    return p


def oracle_run(oracle, sc, steps, seeds=(1, 2, 3)):
    """Runs the oracle restatement on `sc` and on three copies whose initial
    velocity is perturbed by 1e-15 (relative to the mesh size). Returns the
    final state, per-step iterations, and the noise floor (state rel-L2 and
    iteration spread) those perturbations produce."""
    b = oracle.Solid(sc, "port")
    noisy = [oracle.Solid(perturbed(sc, s), "port") for s in seeds]
    it, it_noise = [], [[] for _ in noisy]
    vmax = 0.0
    for _ in range(steps):
        it.append(b.step()["iters"])
        vmax = max(vmax, float(np.linalg.norm(b.state()[1])))
        for c, lst in zip(noisy, it_noise):
            lst.append(c.step()["iters"])
    xb, vb = b.state()
    nx = nv = 0.0
    for c in noisy:
        xc, vc = c.state()
        nx, nv = max(nx, rel(xc, xb)), max(nv, rel(vc, vb))
    spread = max(abs(i - j) for lst in it_noise for i, j in zip(it, lst))
    return {"x": xb, "v": vb, "iters": it, "noise_x": nx, "noise_v": nv, "spread": spread, "vmax": vmax}
