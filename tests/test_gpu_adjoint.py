"""The path-replay adjoint (crt_render_adjoint) against the FP64 CPU
reference gradient of the oracle (same estimator, same Philox samples) and
against central finite differences of the forward renders with common
random numbers (h = 1e-3).

Russian roulette (after the fourth bounce) makes a sample a piecewise
function of kd: its survival test flips when max(throughput) moves past the
sample's random number.  Finite differences with common random numbers see
the smooth part plus the occasional flip (a rare, large jump); the exact-
roulette adjoint is the derivative of the smooth part, so the two agree for
most seeds and differ by a one-sided jump for the few seeds where a flip
falls inside [-h, h].  How often that happens grows with the number of
roulette events a material's factor takes part in: for the wall material,
present in almost every path, differences at 262k paths already sit between
the two adjoint modes, so the depth-6 check uses the parameters the material
inversion optimises (the 32 box albedos, each on few paths) and the light's
emission (roulette does not depend on it).  The default adjoint holds the
survival probability constant instead: unbiased for the expected image, it
is checked against the FP64 reference and, without roulette (depth 3),
against finite differences."""
import numpy as np
import pytest

import oracle
from adjoint_torch import PathTracedImage, material_arrays
from cudart_gb300 import GB300Renderer, GB300Scene, scenes

pytestmark = pytest.mark.gpu


def _adjoint_image(sc, seed=11):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.5, 1.5, (sc.width * sc.height, 3)).astype(np.float32)


def _gpu_adjoint(torch, r, n_mats, adj, spp0, spp, exact=False):
    a4 = torch.zeros((adj.shape[0], 4), dtype=torch.float32, device="cuda")
    a4[:, :3] = torch.from_numpy(adj).cuda()
    gkd = torch.zeros((n_mats, 3), dtype=torch.float32, device="cuda")
    gka = torch.zeros((n_mats, 3), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    r.adjoint(spp0, spp, a4.data_ptr(), gkd.data_ptr(), gka.data_ptr(), exact_roulette=exact)
    r.synchronize()
    return gkd.cpu().numpy().astype(np.float64), gka.cpu().numpy().astype(np.float64)


def _phi(r, adj, spp0, spp):
    r.restart(spp0)
    r.render(spp)
    return float(np.sum(adj.astype(np.float64) * r.accum().astype(np.float64)))


def _significant(ref, frac=1e-3):
    return np.abs(ref) > frac * np.abs(ref).max()


@pytest.mark.parametrize("depth,exact", [(3, False), (6, False), (6, True)])
def test_adjoint_matches_fp64_reference(cuda, depth, exact):
    sc = scenes.material_inversion(width=64, height=64)
    adj = _adjoint_image(sc)
    g = GB300Scene(sc)
    r = GB300Renderer(g, sc.width, sc.height, 16, max_depth=depth, seed=5, mode="wavefront")
    gkd, gka = _gpu_adjoint(cuda, r, len(sc.materials), adj, 0, 16, exact)
    o = oracle.OracleScene(sc)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    rkd, rka = o.adjoint(cam, 5, 16, depth, adj, exact_roulette=exact)
    for got, ref in ((gkd, rkd), (gka, rka)):
        sig = _significant(ref)
        rel = np.abs(got - ref)[sig] / np.abs(ref)[sig]
        assert np.median(rel) < 1e-4 and rel.max() < 1e-2, (np.median(rel), rel.max())
        assert np.all(np.abs(got[~sig]) <= 2e-3 * np.abs(ref).max())


def test_adjoint_matches_finite_differences_without_roulette(cuda):
    # depth 3: Russian roulette starts after the fourth bounce, so the
    # estimator is smooth in kd and ka and CRN differences are exact up to h^2
    sc = scenes.material_inversion(width=128, height=128)
    adj = _adjoint_image(sc)
    g = GB300Scene(sc)
    r = GB300Renderer(g, sc.width, sc.height, 32, max_depth=3, seed=9, mode="wavefront")
    gkd, gka = _gpu_adjoint(cuda, r, len(sc.materials), adj, 0, 32)
    kd0, ka0 = material_arrays(sc)
    h = 1e-3
    checked = 0
    for which, grad, base in (("kd", gkd, kd0), ("ka", gka, ka0)):
        order = np.argsort(-np.abs(grad).ravel())[:6]
        for flat in order:
            m, c = divmod(int(flat), 3)
            vals = []
            for sgn in (1, -1):
                p = base.copy()
                p[m, c] += sgn * h
                g.set_materials(**{which: p})
                vals.append(_phi(r, adj, 0, 32))
            g.set_materials(kd0, ka0)
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(grad[m, c] - fd) <= 0.02 * abs(fd), (which, m, c, grad[m, c], fd)
            checked += 1
    assert checked == 12


def test_exact_roulette_adjoint_matches_finite_differences(cuda):
    sc = scenes.material_inversion(width=64, height=64)
    adj = _adjoint_image(sc)
    g = GB300Scene(sc)
    kd0, ka0 = material_arrays(sc)
    h, spp, seeds = 1e-3, 64, range(8)
    rel = {}
    for seed in seeds:
        r = GB300Renderer(g, sc.width, sc.height, spp, max_depth=6, seed=seed, mode="wavefront",
                          wave_paths=1 << 18)
        gkd, gka = _gpu_adjoint(cuda, r, len(sc.materials), adj, 0, spp, exact=True)
        if seed == 0:   # the largest box-albedo and emission gradients of the first seed
            box = np.abs(gkd[4:]).ravel()
            params = [("kd", 12 + int(f)) for f in np.argsort(-box)[:3]]
            params += [("ka", int(f)) for f in np.argsort(-np.abs(gka).ravel())[:2]]
        for which, flat in params:
            m, c = divmod(flat, 3)
            vals = []
            for sgn in (1, -1):
                p = (kd0 if which == "kd" else ka0).copy()
                p[m, c] += sgn * h
                g.set_materials(**{which: p})
                vals.append(_phi(r, adj, 0, spp))
            g.set_materials(kd0, ka0)
            fd = (vals[0] - vals[1]) / (2 * h)
            grad = (gkd if which == "kd" else gka)[m, c]
            rel.setdefault((which, m, c), []).append((fd - grad) / abs(fd))
    for key, diffs in rel.items():
        print(key, np.round(diffs, 4))
        assert abs(np.median(diffs)) <= 0.02, (key, diffs)


@pytest.mark.parametrize("other", [4, 16])
def test_queue_order_flags_give_the_same_gradient(cuda, other):
    """Octant-binned queues (4) and appending without the window sort (16)
    reorder the paths the replay visits, not the paths themselves."""
    sc = scenes.material_inversion(width=64, height=64)
    adj = _adjoint_image(sc)
    g = GB300Scene(sc)
    out = []
    for flags in (0, other):
        r = GB300Renderer(g, sc.width, sc.height, 8, max_depth=6, seed=2, mode="wavefront", flags=flags,
                          wave_paths=1 << 16)
        out.append(_gpu_adjoint(cuda, r, len(sc.materials), adj, 0, 8))
    for a, b in zip(out[0], out[1]):   # the atomics' order differs: FP32 rounding only
        assert np.allclose(a, b, rtol=1e-4, atol=1e-6 * np.abs(a).max())


def test_torch_autograd_wrapper(cuda):
    torch = cuda
    sc = scenes.material_inversion(width=64, height=64)
    g = GB300Scene(sc)
    r = GB300Renderer(g, sc.width, sc.height, 8, max_depth=6, seed=3, mode="wavefront")
    kd0, ka0 = material_arrays(sc)
    target = torch.rand((sc.width * sc.height, 3), generator=torch.Generator().manual_seed(0))
    kd = torch.tensor(kd0, requires_grad=True)
    ka = torch.tensor(ka0, requires_grad=True)
    img = PathTracedImage.apply(kd, ka, r, 16, 8)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    # the same gradient through the C ABI directly
    adj = (2.0 * (img.detach() - target) / 8).numpy().astype(np.float32)
    gkd, gka = _gpu_adjoint(torch, r, len(sc.materials), adj, 16, 8)
    assert np.allclose(kd.grad.numpy(), gkd, rtol=1e-4, atol=1e-6 * np.abs(gkd).max())
    assert np.allclose(ka.grad.numpy(), gka, rtol=1e-4, atol=1e-6 * np.abs(gka).max())
