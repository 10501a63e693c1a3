"""Grid-file contract between the delta2zreion step and its neighbours: the
input as ReadDeltaFile reads it and the .zreion output as the consumers
(flatskymap, allskymap, limber ReadReionFile) read it, slab by slab."""
import numpy as np
import pytest

from prc_d2z import fields, io


@pytest.mark.parametrize("nproc", [1, 2, 4])
def test_zreion_round_trip_through_consumer_slabs(tmp_path, nproc):
    N = 16
    z = np.abs(fields.gaussian_field(N, 24.0, seed=3)) * 10
    path = str(tmp_path / "run.zreion")
    io.write_zreion_file(path, z)
    assert (tmp_path / "run.zreion").stat().st_size == 4 * N ** 3
    parts = [io.read_reion_file(path, N, nproc, q) for q in range(nproc)]
    back = np.concatenate([p[0] for p in parts], axis=0)
    assert np.array_equal(back, z)
    for q, (s, m) in enumerate(parts):
        assert s.shape == (N // nproc, N, N)
        assert abs(m - float(z[q * (N // nproc):(q + 1) * (N // nproc)].astype(np.float64).mean())) < 1e-9


def test_delta_file_read_matches_written(tmp_path):
    N = 16
    d = fields.gaussian_field(N, 24.0, seed=4)
    path = str(tmp_path / "delta")
    io.write_delta_file(path, d)
    s, mean, sig = io.read_delta_file(path, N)
    assert np.array_equal(s, d)
    assert abs(mean - float(d.astype(np.float64).mean())) < 1e-12
    assert abs(sig - float(np.sqrt((d.astype(np.float64) ** 2).mean()))) < 1e-9


def test_short_file_and_bad_split_are_errors(tmp_path):
    path = str(tmp_path / "short")
    np.zeros(100, np.float32).tofile(path)
    with pytest.raises(IOError):
        io.read_reion_file(path, 16)
    with pytest.raises(ValueError):
        io.read_reion_file(path, 16, nproc=3)
