"""Host BVH construction without a device (gb_bvh_build_stats): the
SAH-optimal 8-wide grouping against the greedy one, bin counts, degenerate
inputs and option errors.  Every tree returned passed the builder's own
structural check (validate_cwbvh: child and triangle ranges, every triangle
referenced exactly once, depth within the traversal stack)."""
import numpy as np
import pytest

from globillum_gb300 import gbpt, scenes


def test_sah_grouping_uses_fewer_nodes(lib_path):
    sc = scenes.icospheres(n_spheres=60, level=3, box=25.0)
    g = gbpt.bvh_build_stats(sc.positions, wide_collapse=2)
    d = gbpt.bvh_build_stats(sc.positions)
    assert g["num_triangles"] == d["num_triangles"] == sc.num_triangles
    assert g["binary_nodes"] == d["binary_nodes"]
    assert d["num_nodes"] < 0.7 * g["num_nodes"]
    assert 1 <= d["depth"] <= 32 and 1 <= g["depth"] <= 32
    # a dearer triangle test keeps more (smaller) leaves and so more nodes
    lo = gbpt.bvh_build_stats(sc.positions, prim_cost=0.15)["num_nodes"]
    hi = gbpt.bvh_build_stats(sc.positions, prim_cost=3.0)["num_nodes"]
    assert lo < hi
    d2 = gbpt.bvh_build_stats(sc.positions)  # deterministic apart from build_ms
    assert {k: v for k, v in d2.items() if k != "build_ms"} == {k: v for k, v in d.items() if k != "build_ms"}


@pytest.mark.parametrize("bins", [2, 16, 32, 64])
def test_bin_counts(lib_path, bins):
    sc = scenes.icospheres(n_spheres=20, level=2, box=12.0)
    st = gbpt.bvh_build_stats(sc.positions, sah_bins=bins)
    assert st["num_triangles"] == sc.num_triangles and st["num_nodes"] >= 1


@pytest.mark.parametrize("n", [1, 2, 3, 4, 9, 100])
def test_small_and_degenerate_inputs(lib_path, n):
    rng = np.random.default_rng(n)
    base = rng.uniform(-1, 1, (n, 9)).astype(np.float32)
    for pos in (base, np.repeat(base[:1], n, axis=0)):
        for wc in (1, 2):
            st = gbpt.bvh_build_stats(pos, wide_collapse=wc)
            assert st["num_triangles"] == n and st["num_nodes"] >= 1


def test_errors(lib_path):
    pos = scenes.cornell().positions.copy()
    bad = pos.copy()
    bad[2, 5] = np.nan
    with pytest.raises(gbpt.GBError) as e:
        gbpt.bvh_build_stats(bad)
    assert e.value.code == gbpt.GB_ERR_INVALID
    for kw in ({"wide_collapse": 3}, {"sah_bins": 1}, {"sah_bins": 65}, {"prim_cost": -1.0}):
        with pytest.raises(gbpt.GBError) as e:
            gbpt.bvh_build_stats(pos, **kw)
        assert e.value.code == gbpt.GB_ERR_INVALID
