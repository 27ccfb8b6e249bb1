"""Host logic of the run loop (no GPU): path interpolation, S control, file formats."""
import numpy as np

from feynsimul_gb300 import pimc_utils as pu


def _reference_interpolation(old, dof, n_new):
    """The index arithmetic of FeynSimul/pimc_utils.py:208-222, written out."""
    walkers = old.shape[0]
    new = np.zeros((walkers, n_new * dof))
    for w in range(walkers):
        for d in range(dof):
            second = d * n_new + np.arange(0, n_new, 2)
            new[w, second] = old[w, second // 2]
            right = second + 2
            right[-1] -= n_new
            new[w, second + 1] = (new[w, second] + new[w, right]) / 2.0
    return new


def test_interpolation_matches_reference_indexing():
    rng = np.random.RandomState(0)
    for dof, n_old in [(1, 8), (3, 16), (6, 4)]:
        old = rng.randn(5, dof * n_old)
        np.testing.assert_allclose(pu.interpolate_paths(old, dof, n_old),
                                   _reference_interpolation(old, dof, 2 * n_old), rtol=0, atol=1e-15)


def test_straight_paths():
    x = np.array([[0.1, -0.2], [0.3, 0.4]])
    p = pu.straight_paths(x, 2, 2, 4)
    assert p.shape == (2, 8)
    assert np.all(p[0, :4] == 0.1) and np.all(p[0, 4:] == -0.2) and np.all(p[1, 4:] == 0.4)


def test_S_control():
    assert pu.clamp_S(1, 4, 8, 512) == 1
    assert pu.clamp_S(1, 64, 1024, 512) == 7          # ceil(log2(64*1024/512))
    assert pu.clamp_S(12, 1, 256, 512) == 8           # log2 N
    assert pu.adapt_S(2, 0.6, 10) == 4
    assert pu.adapt_S(2, 0.3, 10) == 3
    assert pu.adapt_S(2, 0.05, 10) == 1
    assert pu.adapt_S(1, 0.05, 10) == 1
    assert pu.adapt_S(9, 0.9, 10) == 10
    assert pu.adapt_S(3, 0.15, 10) == 3


def test_tsv_and_csv_roundtrip(tmp_path):
    fn = str(tmp_path / "data")
    ops = np.array([[0.5, 0.25, 0.75], [1.0, 2.0, 3.0]])
    pu._output(fn, 16, 1.5, 1234, 0.47, ops, 0.01, 0.002, 20.0, 2)
    pu._output(fn, 32, 2.5, 5678, 0.5, ops * 2, 0.01, 0.002, 20.0, 3)
    text = open(fn + ".tsv").read().splitlines()
    assert text[0] == "#Beta: 20.0"
    assert text[1].startswith("#N\tTime\tpathChanges\tAR\tS\tOperator 0, Walker 0")
    beta, rows, arr = pu.read_tsv(fn + ".tsv")
    assert beta == 20.0 and rows[1] == (32, 2.5, 5678, 0.5, 3)
    np.testing.assert_array_equal(arr[0], ops)
    paths = np.random.RandomState(1).randn(3, 10)
    pu.write_paths_csv(str(tmp_path / "p"), paths)
    np.testing.assert_array_equal(pu.read_paths_csv(str(tmp_path / "p"), 3, 10), paths)
