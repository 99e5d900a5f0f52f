"""The oracle's intersector (the Embree-semantics closest hit every GPU parity
test compares against): its BVH2 traversal gives the brute-force answer --
the same primitive, or one at exactly the same distance, and bit-identical t --
on seeded rays, including rays from surfaces with tnear 0.001, axis-aligned
rays and rays that start inside the scene's bounds."""
import numpy as np
import pytest

import lantern_gb300.scenes as S
from oracle import oracle as O

MISS = 0xFFFFFFFF


def _rays(lo, hi, n, seed):
    rays = S.random_rays(n, lo, hi, seed=seed)
    rng = np.random.default_rng(seed + 1)
    k = n // 4  # axis-aligned directions
    axis = rng.integers(0, 3, k)
    rays[:k, 4:7] = 0.0
    rays[np.arange(k), 4 + axis] = rng.choice([-1.0, 1.0], k)
    rays[k:2 * k, 3] = 0.001  # tnear as for secondary rays
    return rays


@pytest.mark.parametrize("make", [
    lambda: S.nine_spheres(width=16, height=16, slices=24, stacks=12, name="obvh_nine"),
    lambda: S.displaced_icosphere_scene(width=16, height=16, levels=4, name="obvh_ico4"),
    lambda: S.procedural_scene(width=16, height=16, name="obvh_proc"),
])
def test_oracle_bvh_equals_brute_force(scene_dir, make):
    orc = O.OracleScene(make().write(scene_dir))
    rays = _rays(np.array([-2.0, 0.02, -2.0]), np.array([2.0, 2.0, 2.0]), 4096, seed=21)
    b = orc.intersect(rays, use_bvh=True)
    f = orc.intersect(rays, use_bvh=False)
    hit = f[:, 3] != MISS
    assert hit.sum() > 500
    assert np.array_equal(b[:, 3] == MISS, ~hit)
    assert np.array_equal(b[hit, 0], f[hit, 0])  # t, as float bits
    same = b[:, 3] == f[:, 3]
    assert np.all(same | ~hit)  # the same primitive (ties are bit-equal t, checked above)
