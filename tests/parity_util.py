"""Shared helpers for the GPU parity tests."""
import copy

import numpy as np


# Every calibrated comparison of the run: (test case, quantity, measured,
# bar used, oracle floor). conftest prints them at the end of the session so
# the effective bars are visible in the test log.
BARS = []


def bar_cap(sc):
    """Largest bar a calibrated comparison may use for scene `sc`: 100 x its
    CG relative tolerance, at least 1e-6. CG stops on |r| <= rel |r0|, so when
    a 1e-15 input change moves the stopping iteration by one the state moves
    by about the tolerance times the conditioning; the oracle's own floor is
    then of that order, and a floor far above it means something else moved."""
    return max(1e-6, 100.0 * float(sc.rel_eps))


def check_bar(case, quantity, measured, tol, floor, cap=1e-6, mult=10.0):
    """Asserts measured <= max(tol, 10 x floor), the bar of the calibrated
    comparisons, and that this bar stays within `cap` (bar_cap of the scene):
    an oracle floor that grew (a regression that would otherwise pass inside
    an inflated bar) fails the test instead of widening it silently. Records
    the figures."""
    bar = max(tol, mult * floor)
    BARS.append((case, quantity, float(measured), float(bar), float(floor)))
    assert bar <= max(cap, tol), \
        f"{case} {quantity}: bar {bar:.3g} from the oracle floor {floor:.3g} exceeds the cap {cap:.3g}"
    assert measured <= bar, f"{case} {quantity}: {measured:.3g} > bar {bar:.3g} (floor {floor:.3g})"
    return bar


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
