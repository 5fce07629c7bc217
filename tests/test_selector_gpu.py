"""AUTO chooses the variant from sampled statistics, not from sizes alone.

Three inputs of the same size (100,000 x 100,000 points, inside the band
where the selector samples) lead to three different variants when the
early-break threshold is set, as the reference's -eb_only_threshold sets it:

  duplicated 3-D points  the sampled early-break scans stop after a few
                         pairs (small mean count)        -> early break
  uniform 2-D points     no query outside the target's box, occupancy skew
                         ~1                              -> uniform grid
  clustered 3-D points   occupancy skew far above 1      -> LBVH

With the tuned table's own threshold (0: on this GPU the early break lost to
the LBVH above the small-size band on every swept input, duplicated data
included) the statistics still pick between the grid and the LBVH.  Every
result is checked against the oracle as in the parity suite.  This is the
role of the reference's hybrid decision (src/hd_impl/
hausdorff_distance_hybrid.h:143-199), which picks EB-only or the index from
sampled iteration counts.
"""
import numpy as np
import pytest

import hd_oracle
from hausdorffdistance_gb300 import autotune, synth

pytestmark = pytest.mark.gpu

N = 100_000


def check(a, b, r, undirected=False):
    want = hd_oracle.hd_f32(a, b, undirected=undirected)
    assert np.float32(r.hd_f32) == want["hd_f32"]
    src, dst = (a, b) if r.direction == 0 else (b, a)
    assert hd_oracle.dist2_f32(src[int(r.ia)], dst[int(r.ib)]) == want["d2"]


def inputs():
    dup = autotune.duplicated3d(N, seed=5)
    rng = np.random.default_rng(6)
    uni = (rng.random((N, 2)).astype(np.float32), rng.random((N, 2)).astype(np.float32))
    clu = synth.clusters3d(N, seed=7)
    return (("dup", dup), ("uniform", uni), ("clusters", clu))


@pytest.mark.parametrize("eb_threshold", [64, 0])
def test_auto_picks_variants_from_statistics(eb_threshold):
    import hausdorffdistance_gb300 as hd
    got = {}
    with hd.Engine(device=0, eb_only_threshold=eb_threshold) as eng:
        for name, (a, b) in inputs():
            r = eng.solve(a, b, variant="auto")
            got[name] = hd._lib.VARIANT_NAMES[r.variant_used]
            check(a, b, r)
            assert r.sample_mean[0] > 0 and r.grid_skew[0] > 0
            if name == "dup":
                assert r.sample_mean[0] <= 128
            if name == "uniform":
                assert r.grid_outside[0] == 0.0 and r.grid_skew[0] < 1.5
                assert r.sample_mean[0] > 1000
            if name == "clusters":
                assert r.grid_skew[0] > 10.0
    want_dup = "eb" if eb_threshold else "lbvh"
    assert got == {"dup": want_dup, "uniform": "grid", "clusters": "lbvh"}


def test_auto_undirected_shares_the_lbvh_unless_both_directions_qualify(engine):
    import hausdorffdistance_gb300 as hd
    # B has 5% outliers outside A's box: B->A does not qualify for the grid,
    # so both directions take the fused LBVH.
    a, b = synth.uniform2d(N, seed=8)
    r = engine.solve(a, b, undirected=True, variant="auto")
    assert r.grid_outside[1] > 0.002
    assert (r.variant_used, r.variant_used_ba) == (hd._lib.VARIANT_LBVH, hd._lib.VARIANT_LBVH)
    check(a, b, r, undirected=True)
    # Two independent uniform draws: both directions qualify.
    rng = np.random.default_rng(9)
    a = rng.random((N, 2)).astype(np.float32)
    b = rng.random((N, 2)).astype(np.float32)
    r = engine.solve(a, b, undirected=True, variant="auto")
    assert (r.variant_used, r.variant_used_ba) == (hd._lib.VARIANT_GRID, hd._lib.VARIANT_GRID)
    check(a, b, r, undirected=True)
