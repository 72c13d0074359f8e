"""XTR distribution checkpoints written and read by the C ABI, byte for byte against
the extraction-file oracle, and a restart that continues bit-exactly."""
import numpy as np
import pytest

from hemelb_gb300 import capi, cases
from oracle import xtr as X

pytestmark = pytest.mark.gpu

ORIGIN = (0.034, 0.001, 0.074)


def bifurcation():
    return cases.bifurcation(seed=5, parent_radius=8.0, parent_length=40.0, daughter_length_factor=1.2, period=200.0)


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32DEV])
def test_checkpoint_bytes_offsets_append_and_restart(tmp_path, precision):
    """FP64: the restart continues bit for bit.  FP32 deviations: the file holds
    f = g + w in double, which keeps the FP32 deviation g exactly except where
    |g| is below ~2^-29 w (its low bits fall off the sum), so the restart reads
    back the same f and continues within 1e-9."""
    c = bifurcation()
    s = c.solver(precision)
    s.SetInitialConditions()
    s.DoTimeStep(9)
    path = str(tmp_path / "state.xtr")
    s.WriteCheckpoint(path, 9, voxel_size=0.3e-3, origin=ORIGIN)
    coords, f9 = s.site_coords(), s.GetFOld()
    n = len(coords)
    head = X.checkpoint_header(n, 0.3e-3, ORIGIN)
    rec9 = X.checkpoint_record(9, coords, f9)
    assert open(path, "rb").read() == head + rec9
    assert (tmp_path / "state.off").read_bytes() == X.offset_file(len(head), len(rec9))
    s.DoTimeStep(4)
    s.WriteCheckpoint(path, 13, voxel_size=0.3e-3, origin=ORIGIN, append=True)
    f13 = s.GetFOld()
    _, recs = X.read_checkpoint(open(path, "rb").read())
    assert [r[0] for r in recs] == [9, 13]
    # the reader's binary search needs increasing timesteps: an append that would
    # repeat or go back is refused and leaves the file as it was
    before = open(path, "rb").read()
    for t in (13, 11, 0):
        with pytest.raises(RuntimeError, match="does not follow"):
            s.WriteCheckpoint(path, t, voxel_size=0.3e-3, origin=ORIGIN, append=True)
    assert open(path, "rb").read() == before
    assert np.array_equal(recs[1][2], f13) and np.array_equal(recs[1][1], coords)
    # restart from step 9 in a fresh solver: both time levels hold the record,
    # and four more steps reproduce the original run bit for bit
    r = c.solver(precision)
    assert r.ReadCheckpoint(path, 9) == 9
    assert np.array_equal(r.GetFOld(), f9) and np.array_equal(r.GetFNew(), f9)
    r.SetTimeStep(10)
    r.DoTimeStep(4)
    if precision == capi.FP64:
        assert np.array_equal(r.GetFOld(), f13)
    else:
        assert np.abs(r.GetFOld() - f13).max() <= 1e-9
    assert r.ReadCheckpoint(path) == 13  # the last record by default
    assert np.array_equal(r.GetFOld(), f13)


def test_checkpoint_reader_rejects_other_files(tmp_path):
    c = bifurcation()
    s = c.solver()
    s.SetInitialConditions()
    path = str(tmp_path / "a.xtr")
    s.WriteCheckpoint(path, 1)
    with pytest.raises(RuntimeError):
        s.ReadCheckpoint(path, 2)  # no such timestep
    coords = s.site_coords()
    f = s.GetFOld()
    moved = coords.copy()
    moved[3, 0] += 1  # a site that is not this geometry's
    bad = str(tmp_path / "b.xtr")
    open(bad, "wb").write(X.checkpoint_header(len(coords)) + X.checkpoint_record(1, moved, f))
    with pytest.raises(RuntimeError):
        s.ReadCheckpoint(bad)
    short = str(tmp_path / "c.xtr")
    open(short, "wb").write(X.checkpoint_header(len(coords) - 1) + X.checkpoint_record(1, coords[1:], f[1:]))
    with pytest.raises(RuntimeError):
        s.ReadCheckpoint(short)
    # a file written by the oracle loads exactly
    good = str(tmp_path / "d.xtr")
    g = f * (1.0 + 1e-3)
    open(good, "wb").write(X.checkpoint_header(len(coords)) + X.checkpoint_record(7, coords, g))
    assert s.ReadCheckpoint(good) == 7
    assert np.array_equal(s.GetFOld(), g)


def test_checkpoint_of_a_geometry_larger_than_one_write_chunk(tmp_path):
    """A pipe of ~125k sites: the record is encoded, written and read back in
    several chunks of sites; the bytes equal the oracle's and the state returns."""
    c = cases.pipe(radius=20.0, length=100)
    s = c.solver()
    s.SetInitialConditions()
    s.DoTimeStep(5)
    assert s.n_sites > 65536  # two chunks or more
    path = str(tmp_path / "big.xtr")
    s.WriteCheckpoint(path, 5)
    coords, f = s.site_coords(), s.GetFOld()
    assert open(path, "rb").read() == X.checkpoint_header(len(coords)) + X.checkpoint_record(5, coords, f)
    r = c.solver()
    assert r.ReadCheckpoint(path) == 5
    assert np.array_equal(r.GetFOld(), f)
