"""Size-independent properties of the full-size icosphere render: 1,310,724
triangles, 1024x1024, 64 samples per pixel, depth 10, roulette after bounce 3
(the benchmark's frame), which the oracle cannot render in test time.

* Every pixel gets exactly 64 samples and nothing in the film is NaN or
  infinite (no sample contributed a non-finite value).
* The render is linear in its samples: frames 0-31 plus frames 32-63 equal
  frames 0-63 -- sample counts and path lengths exactly, colour sums within the
  reordering of float atomics -- because each sample's sampler is keyed by
  (pixel, frame) alone. With the library's default wavefront (16,777,216 paths
  in flight, fewer than the 67,108,864 samples) finished paths are replaced by
  new work items inside the loop, so this also checks that no work item is lost
  or taken twice.
"""
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene

pytestmark = pytest.mark.gpu


def test_full_size_render_counts_finiteness_and_linearity(scene_dir):
    path = S.ensure_written(S.displaced_icosphere_scene(name="full_icosphere"), scene_dir)
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    assert (sc.width, sc.height) == (1024, 1024)
    full = FrameBuffer(sc.width, sc.height, "cuda:0")
    whole = Integrator(sc, full, max_depth=10, rr_depth=3)
    whole.RenderFrame(64)
    st = whole.stats()
    halves = FrameBuffer(sc.width, sc.height, "cuda:0")
    two = Integrator(sc, halves, max_depth=10, rr_depth=3)
    two.RenderFrame(32)
    two.RenderFrame(32)
    torch.cuda.synchronize()

    assert st.samples == 1024 * 1024 * 64 and st.nonfinite_samples == 0
    for fb in (full, halves):
        assert int(fb.ColorSampleCount.min()) == 64 and int(fb.ColorSampleCount.max()) == 64
        assert bool(torch.isfinite(fb.ColorData).all())
    assert torch.equal(halves.Bounces, full.Bounces)
    # colour sums are sums of non-negative terms (at most ~1,300 per pixel), so a
    # different order of the float additions moves them by well under 2e-4
    assert torch.allclose(halves.ColorData, full.ColorData, rtol=2e-4, atol=1e-6)
    a, b = float(full.ColorData.double().sum()), float(halves.ColorData.double().sum())
    assert a > 0 and abs(a - b) <= 1e-5 * a
