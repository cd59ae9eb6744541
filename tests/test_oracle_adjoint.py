"""The oracle's FP64 reference gradient (orc_adjoint) against central finite
differences of the oracle's own forward renders with common random numbers.
Depth 3 keeps Russian roulette out (it starts after the fourth bounce), so
the estimator is a smooth function of kd and ka and the two must agree to
the finite-difference error."""
import dataclasses

import numpy as np

import oracle
from cudart_gb300 import scenes

H = 1e-3


def _phi(sc, cam, adj, depth, lights):
    o = oracle.OracleScene(sc, lights=lights)
    acc, _, _ = o.render(cam, seed=7, spp=16, max_depth=depth)
    return float(np.sum(adj.astype(np.float64) * acc.astype(np.float64)))


def _with(sc, m, field, c, d):
    mats = list(sc.materials)
    v = list(getattr(mats[m], field))
    v[c] += d
    mats[m] = dataclasses.replace(mats[m], **{field: tuple(v)})
    return dataclasses.replace(sc, materials=mats)


def test_reference_gradient_matches_finite_differences():
    sc = scenes.material_inversion(width=40, height=40)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    adj = np.random.default_rng(0).uniform(0.5, 1.5, (sc.width * sc.height, 3)).astype(np.float32)
    lights = sc.light_indices()
    gkd, gka = oracle.OracleScene(sc).adjoint(cam, 7, 16, 3, adj)
    light_mat = int(sc.material_ids[lights[0]])
    cases = [("kd", m, c, gkd) for m in (5, 9, 20) for c in range(3)]
    cases += [("ka", light_mat, c, gka) for c in range(3)]
    for field, m, c, grad in cases:
        fd = (_phi(_with(sc, m, field, c, H), cam, adj, 3, lights) -
              _phi(_with(sc, m, field, c, -H), cam, adj, 3, lights)) / (2 * H)
        assert abs(grad[m, c] - fd) <= 2e-3 * abs(fd), (field, m, c, grad[m, c], fd)


def test_zero_adjoint_gives_zero_gradient():
    sc = scenes.material_inversion(width=16, height=16)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    gkd, gka = oracle.OracleScene(sc).adjoint(cam, 1, 4, 6, np.zeros((256, 3), np.float32))
    assert not gkd.any() and not gka.any()


def test_exact_roulette_gradient_matches_finite_differences_per_seed():
    # depth 6: with the roulette renormalisation differentiated, each seed's
    # gradient equals its central difference unless a roulette decision flips
    # inside [-h, h] (a rare one-sided jump), so the median over seeds agrees
    sc = scenes.material_inversion(width=40, height=40)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    adj = np.random.default_rng(2).uniform(0.5, 1.5, (sc.width * sc.height, 3)).astype(np.float32)
    lights = sc.light_indices()

    def phi(s, seed):
        acc, _, _ = oracle.OracleScene(s, lights=lights).render(cam, seed=seed, spp=32, max_depth=6)
        return float(np.sum(adj.astype(np.float64) * acc.astype(np.float64)))

    for m, c in ((5, 0), (9, 1)):
        diffs = []
        for seed in range(6):
            gkd, _ = oracle.OracleScene(sc).adjoint(cam, seed, 32, 6, adj, exact_roulette=True)
            fd = (phi(_with(sc, m, "kd", c, H), seed) - phi(_with(sc, m, "kd", c, -H), seed)) / (2 * H)
            diffs.append((fd - gkd[m, c]) / abs(fd))
        assert abs(np.median(diffs)) <= 0.01, (m, c, np.round(diffs, 4))
