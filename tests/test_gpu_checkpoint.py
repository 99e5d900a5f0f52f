"""Checkpoint / resume of a progressive render: the film and the next frame
number are the whole state, so a render interrupted, saved, restored and
continued takes exactly the samples of an uninterrupted one."""
import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene

pytestmark = pytest.mark.gpu


def test_resume_continues_the_same_samples(scene_dir, tmp_path):
    sc = Scene(0)
    sc.LoadSceneFromJSON(S.tiny_scene(width=40, height=32, name="ckpt_tiny").write(scene_dir))
    whole = Integrator(sc, FrameBuffer(sc.width, sc.height, "cuda:0"), max_depth=10)
    whole.RenderFrame(7)
    part = Integrator(sc, FrameBuffer(sc.width, sc.height, "cuda:0"), max_depth=10)
    part.RenderFrame(3)
    part.checkpoint(str(tmp_path / "film.npz"))
    resumed = Integrator.resume(sc, str(tmp_path / "film.npz"), max_depth=10)
    assert resumed.frame_number == 3
    resumed.RenderFrame(4)
    torch.cuda.synchronize()
    a, b = whole.frame_buffer, resumed.frame_buffer
    assert torch.equal(a.ColorSampleCount, b.ColorSampleCount)
    assert torch.equal(a.Bounces, b.Bounces)
    x, y = a.ColorData.double(), b.ColorData.double()
    assert float((x - y).abs().max()) <= 1e-5 * (float(x.abs().max()) + 1e-30)
    assert resumed.frame_number == whole.frame_number == 7
