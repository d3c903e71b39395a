"""Host-side checks of the tensor-core contraction's plan (no GPU): for
triangle lists of the reference's loop (pyspectrum.py:415-417) and for
shuffled / thinned / relabelled lists, every triangle must be read at exactly
one (pair row, column) cell whose shells are the triangle's, and each row's
shells must agree with the producer threads' table
(pyspec_bk_plan_check).  Which plan a list gets (runs of the two largest
shells, or a pair cover on three tiles) is asserted where it sets the MMA
count of the bench workload."""
import numpy as np
import pytest

from pyspectrum_gb300 import _lib, core


def plan_check(nshell, tri):
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    info = np.zeros(10, dtype=np.int64)
    _lib.call("pyspec_bk_plan_check", int(nshell), tri.ctypes.data, int(tri.shape[1]), info.ctypes.data, 10)
    return dict(zip(["groups", "tiles", "cover", "mma", "slots", "wide", "macs", "clashes", "chunk", "bwarps"],
                    info.tolist()))


@pytest.mark.parametrize("nmax", [1, 2, 10, 20, 30, 36, 40, 45, 60, 64])
def test_reference_loop_plans(nmax):
    tri = core.triangles(1, nmax) - 1
    info = plan_check(nmax, tri)
    assert info["groups"] >= 1 and info["tiles"] in (2, 3, 4)


def test_bench_workload_gets_three_tiles():
    """Nmax 40 (6350 triangles): 372 rows of a pair cover fit 3 tiles, so
    12 MMAs per 32 voxels instead of 16 (440 (largest, middle) pairs need 4);
    Nmax 30 fits 2."""
    info = plan_check(40, core.triangles(1, 40) - 1)
    assert info == {"groups": 1, "tiles": 3, "cover": 1, "mma": 12, "slots": info["slots"], "wide": 1,
                    "macs": 3 * 128 * 2 * 2 * 40, "clashes": info["clashes"], "chunk": 64, "bwarps": 1}
    # producer threads that share load phases are paired to avoid bank clashes
    # (32 phase pairs x up to 8 loads; unpaired greedy order gave ~10x more)
    assert info["clashes"] <= 16
    # Nmax 30: 38 row threads of runs need 4 tiles; 32 two-slot cover blocks fit 2
    info30 = plan_check(30, core.triangles(1, 30) - 1)
    assert info30["cover"] == 1 and info30["tiles"] == 2 and info30["mma"] == 8
    # 64-voxel chunks for both; B-operand writer warps only with three tiles
    assert info30["chunk"] == 64 and info30["bwarps"] == 0
    # Nmax 20: runs already fit 2 tiles, no cover is searched
    info20 = plan_check(20, core.triangles(1, 20) - 1)
    assert info20["cover"] == 0 and info20["tiles"] == 2


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_shuffled_and_relabelled_lists(seed):
    rng = np.random.default_rng(seed)
    nmax = 40
    tri = core.triangles(1, nmax) - 1
    # thin, shuffle the triangle order and the slot order within triangles
    keep = rng.random(tri.shape[1]) < [1.0, 0.7, 0.3][seed]
    tri = tri[:, keep][:, rng.permutation(int(keep.sum()))]
    for t in range(tri.shape[1]):
        tri[:, t] = tri[rng.permutation(3), t]
    plan_check(nmax, tri)
    # shells relabelled by a permutation: a different but equally valid plan
    perm = rng.permutation(nmax)
    plan_check(nmax, perm[tri])


def test_arbitrary_lists_with_repeated_shells():
    rng = np.random.default_rng(7)
    nshell = 24
    seen, cols = set(), []
    while len(cols) < 1500:
        t = tuple(sorted(rng.integers(0, nshell, 3).tolist()))
        if t not in seen:
            seen.add(t)
            cols.append(t)
    plan_check(nshell, np.array(cols, dtype=np.int32).T)


def test_repeated_triangle_rejected():
    tri = core.triangles(1, 12) - 1
    tri = np.concatenate([tri, tri[:, [5]][[2, 0, 1]]], axis=1)   # triangle 5 again, slots reordered
    with pytest.raises(_lib.PyspecError, match="repeats"):
        plan_check(12, tri)


def test_out_of_range_shell_rejected():
    tri = core.triangles(1, 12) - 1
    with pytest.raises(_lib.PyspecError, match="outside"):
        plan_check(11, tri)
