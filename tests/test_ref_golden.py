"""The oracle against the reference implementation's own outputs.

The golden fixtures tests/golden/ref_*.npz were made by running the reference
(pcdslab/gpu-sfft, built from its own sources) on a GPU with
tests/golden/make_ref_fixtures.py.  These tests need no GPU: they pin the CPU
oracle, which the GPU tests then use as their checker, to the reference.
"""
import numpy as np
import pytest

import _refparity as RP


@pytest.mark.parametrize("case", RP.STAGE_CASES)
def test_oracle_matches_reference_stage(O, case):
    """Each reference stage function (innerLoop.h:32-50) on race-free inputs."""
    meta, inp, ref = RP.load_stage(case)
    got = RP.oracle_stage(O, RP.kind_of(case), meta, inp)
    RP.check_stage(RP.kind_of(case), got, ref)
    if case == "rlfc":
        assert got["offset"] == ref["offset"]  # drand48 draw of innerLoop.cu:123


@pytest.mark.parametrize("name", RP.E2E_FIXTURES)
def test_oracle_matches_reference_end_to_end(O, name):
    """Whole outer_loop (outerLoop.cu:65-190) with the reference's own signal,
    filter and glibc draws: same candidate set, values within 1e-12, same
    top-k location set."""
    f = RP.load_e2e(O, name)
    reps = f["reps"]
    assert reps[0] == reps[1] == reps[2]  # the reference agrees with itself here
    offs, a, ai = f["draws"]
    o = O.outer_loop(f["x"], f["p"], f["ft_dropped"], f["ff"], offs, a, ai, floor_rel=0.0)
    assert o["status"] == 0
    RP.compare_e2e(RP.as_dict(o["nodes"]), reps[0], f["p"].k, 1e-12)


def test_reference_loses_its_residue_taps(O):
    """permFilterTillKernel's residue thread (innerLoop.cu:745-754) adds into
    bins that the bucket threads are still updating without atomics; at these
    sizes its additions are overwritten.  The code as written (the residue
    quirk) therefore does not give the reference's values, while the same run
    without the residue taps does."""
    f = RP.load_e2e(O, "ref_n16_k50_s1")
    offs, a, ai = f["draws"]
    ref = f["reps"][0]
    as_written = RP.as_dict(O.outer_loop(f["x"], f["p"], f["ft"], f["ff"], offs, a, ai,
                                         quirks=O.QUIRK_RESIDUE, floor_rel=0.0)["nodes"])
    dropped = RP.as_dict(O.outer_loop(f["x"], f["p"], f["ft_dropped"], f["ff"], offs, a, ai,
                                      floor_rel=0.0)["nodes"])
    common = [k for k in ref if k in as_written]
    rel_written = np.median([abs(as_written[k] - ref[k]) / abs(ref[k]) for k in common])
    rel_dropped = max(abs(dropped[k] - ref[k]) / abs(ref[k]) for k in ref)
    assert rel_written > 1e-6 and rel_dropped < 1e-10


@pytest.mark.parametrize("name", RP.E2E_FIXTURES[::2])
def test_oracle_filter_matches_reference(O, name):
    """Filter design (make_multiple_t, cuExperiment.cu:277-448).  The
    reference builds the boxcar and the phase ramp by running sums over n
    (:389-420); the oracle's recurrence mode follows that to 1e-11, its exact
    form stays within the reference's own accumulated rounding (1e-10)."""
    f = RP.load_e2e(O, name)
    p = f["p"]
    n, B = p.n, p.B
    half = n // (2 * B)
    win = np.r_[0:half + 1, n - half:n]
    ft_r, ffw_r = f["ft"], f["ff_win"]
    for quirks, tol in ((O.QUIRK_FILTER_RECURRENCE, 1e-11), (0, 1e-10)):
        ft, ff = O.design_filter(p, quirks=quirks)
        assert np.abs(ft - ft_r).max() <= tol * np.abs(ft_r).max()
        assert np.abs(ff[win] - ffw_r).max() <= tol * np.abs(ffw_r).max()
