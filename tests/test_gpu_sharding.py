"""Sample sharding on the library's own output (one GPU standing in for the
ranks, one after another).

Two renderers take the sample ranges cudart_gb300.sharding.sample_range
gives ranks 0 and 1 of a frame (crt_render_restart(s0)), and their FP32
accumulators are summed as the all_reduce of a two-rank run would sum them
(through the zero-copy accumulator tensors the bench's ranks reduce).  The
sum must equal the single render of all samples up to FP32 rounding: the
shards add the same per-sample radiances in a different grouping.  For n
non-negative terms each order's sum is within (n-1) u of the exact sum
(u = 2^-24), so two orders of 24 terms differ by at most about 2.8e-6
relative per pixel.
"""
import numpy as np
import pytest

from cudart_gb300 import GB300Renderer, GB300Scene, scenes
from cudart_gb300.sharding import sample_range

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["megakernel", "wavefront"])
@pytest.mark.parametrize("world", [2, 3])
def test_sample_shards_sum_to_the_single_render(cuda, mode, world):
    torch = cuda
    sc = scenes.mixed_mid(width=160, height=90, subdiv=3)
    g = GB300Scene(sc)
    spp = 24
    single = GB300Renderer(g, sc.width, sc.height, spp, max_depth=8, seed=99, mode=mode)
    single.render(spp)
    ref = single.accum().astype(np.float64)
    total = torch.zeros((sc.width * sc.height, 4), dtype=torch.float32, device="cuda")
    for rank in range(world):
        s0, s1 = sample_range(spp, rank, world)
        r = GB300Renderer(g, sc.width, sc.height, s1 - s0, max_depth=8, seed=99, mode=mode)
        r.restart(s0)
        r.render(s1 - s0)
        r.synchronize()
        total += r.accum_tensor()          # what all_reduce(SUM) forms across ranks
        del r
    got = total[:, :3].cpu().numpy().astype(np.float64)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
    assert rel.max() <= 3e-6, rel.max()
    assert float(np.sum((got - ref) ** 2) / np.sum(ref ** 2)) <= 1e-12
