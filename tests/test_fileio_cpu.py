"""Graph-file input (gg_read_rb / gg_read_edgelist): host code of the library, no GPU.

Rutherford-Boeing files are checked against scipy's Harwell-Boeing writer (the same card
layout without right-hand sides) and against hand-written files covering what Fortran
fixed-width formats allow (fields that touch, D exponents, a dropped E, scale factors,
symmetric / pattern / skew storage); edge lists against the adjacency they describe."""
import numpy as np
import pytest
import scipy.io
import scipy.sparse as sp

import gpugraphs as G
from gpugraphs import fileio


@pytest.fixture(scope="module", autouse=True)
def built():
    from gpugraphs import _lib
    import os
    if not os.path.exists(_lib.LIB_PATH):
        import build_lib
        build_lib.build()


def test_rb_matches_scipy_hb_writer(tmp_path):
    A = sp.random(57, 43, density=0.08, format="csc", random_state=np.random.default_rng(2))
    A.data = A.data * 1e3 - 400.0
    path = tmp_path / "a.rb"
    scipy.io.hb_write(str(path), A)
    B = fileio.read_rb(str(path))
    assert B.shape == A.shape
    A.sort_indices()
    assert np.array_equal(B.indptr, A.indptr) and np.array_equal(B.indices, A.indices)
    assert np.array_equal(B.data, A.data)


def test_rb_fixed_width_symmetric_pattern(tmp_path):
    # 4x4 symmetric pattern, lower triangle stored; (4I2) fields touch once ids reach 10
    txt = ("lower triangle of a 4x4 pattern                                         KEY\n"
           "             4             1             1             0\n"
           "psa                        4             4             6             0\n"
           "(5I2)           (6I2)\n"
           " 1 3 5 6 7\n"
           " 1 2 3 4 3 4\n")
    path = tmp_path / "p.rb"
    path.write_text(txt)
    data = fileio.RBData(str(path))
    assert data.kind & fileio.PATTERN and data.kind & fileio.SYMMETRIC
    D = data.data.toarray()
    want = np.array([[1, 1, 0, 0], [1, 0, 1, 1], [0, 1, 1, 0], [0, 1, 0, 1]], float)
    assert np.array_equal(D, want)
    tri = fileio.read_rb(str(path), expand_symmetric=False).toarray()
    assert np.array_equal(tri, np.tril(want))


def test_rb_touching_fields_and_fortran_reals(tmp_path):
    # 12x2 matrix: row indices 10, 11, 12 written without separators in (3I2)
    txt = ("touching fields                                                         KEY2\n"
           "             5             1             1             2\n"
           "rua                       12             2             4             0\n"
           "(3I2)           (3I2)           (1P,3D12.4)\n"
           " 1 3 5\n"
           "101112\n"
           " 1\n"
           "  1.5000D+02 -2.2500-003  7.0000E+00\n"
           "  4.0000D-01\n")
    path = tmp_path / "t.rb"
    path.write_text(txt)
    B = fileio.read_rb(str(path)).toarray()
    assert B.shape == (12, 2)
    assert B[9, 0] == 150.0 and B[10, 0] == -2.25e-3
    assert B[11, 1] == 7.0 and B[0, 1] == 0.4


def test_rb_skew_and_errors(tmp_path):
    txt = ("skew                                                                    KEY3\n"
           "             4             1             1             1\n"
           "rza                        3             3             2             0\n"
           "(4I3)           (4I3)           (4E12.4)\n"
           "  1  3  3  3\n"
           "  2  3\n"
           "  2.0000E+00  5.0000E-01\n")
    path = tmp_path / "z.rb"
    path.write_text(txt)
    D = fileio.read_rb(str(path)).toarray()
    assert np.array_equal(D, np.array([[0, -2, -0.5], [2, 0, 0], [0.5, 0, 0]]))
    with pytest.raises(G.ArgumentError):
        fileio.read_rb(str(tmp_path / "missing.rb"))
    cpx = txt.replace("rza", "cua")
    (tmp_path / "c.rb").write_text(cpx)
    with pytest.raises(G.UnsupportedError):
        fileio.read_rb(str(tmp_path / "c.rb"))
    bad = txt.replace("  1  3  3  3", "  1  4  3  3")
    (tmp_path / "b.rb").write_text(bad)
    with pytest.raises(G.ArgumentError):
        fileio.read_rb(str(tmp_path / "b.rb"))
    # a middle pointer far beyond nnz + 1: rejected before any entry is read through it
    far = txt.replace("  1  3  3  3", "  1999  3  3")
    (tmp_path / "f.rb").write_text(far)
    with pytest.raises(G.ArgumentError, match="column pointers"):
        fileio.read_rb(str(tmp_path / "f.rb"))


def test_edgelist_to_transposed_adjacency(tmp_path):
    txt = ("# a small directed graph\n"
           "1 2\n"
           "% another comment\n"
           "2,3\n"
           "3\t1\n"
           "1 2\n"      # repeated edge: ignored
           "4 4\n")     # self loop kept
    path = tmp_path / "g.txt"
    path.write_text(txt)
    AT, weighted = fileio.read_edgelist(str(path))
    assert not weighted and AT.shape == (4, 4)
    A = AT.T.toarray()
    want = np.zeros((4, 4))
    for u, v in ((1, 2), (2, 3), (3, 1), (4, 4)):
        want[u - 1, v - 1] = 1
    assert np.array_equal(A, want)
    w = tmp_path / "w.txt"
    w.write_text("0 1 2.5\n1 2 0.25\n0 1 9.0\n")
    AT, weighted = fileio.read_edgelist(str(w), base=0)
    assert weighted and AT.shape == (3, 3)
    assert AT[1, 0] == 2.5 and AT[2, 1] == 0.25 and AT.nnz == 2
    with pytest.raises(G.ArgumentError):
        fileio.read_edgelist(str(w), base=1)
    (tmp_path / "x.txt").write_text("1 x\n")
    with pytest.raises(G.ArgumentError):
        fileio.read_edgelist(str(tmp_path / "x.txt"))


def test_mtx_matches_scipy_writer(tmp_path):
    rng = np.random.default_rng(7)
    A = sp.random(40, 33, density=0.1, format="coo", random_state=rng)
    A.data = A.data * 100 - 30
    path = tmp_path / "a.mtx"
    scipy.io.mmwrite(str(path), A, precision=17)
    B = fileio.read_mtx(str(path))
    assert B.shape == A.shape
    assert np.array_equal(B.toarray(), A.toarray())
    # symmetric integer storage: the lower triangle written, both read back
    S = sp.random(25, 25, density=0.2, format="csr", random_state=rng)
    S = (S + S.T).tocoo()
    S.data = np.round(S.data * 10) + 1
    p2 = tmp_path / "s.mtx"
    scipy.io.mmwrite(str(p2), S.astype(np.int64), symmetry="symmetric")
    D = fileio.read_mtx(str(p2)).toarray()
    assert np.array_equal(D, S.toarray())
    tri = fileio.read_mtx(str(p2), expand_symmetric=False).toarray()
    assert np.array_equal(tri, np.tril(S.toarray()))


def test_mtx_pattern_skew_and_errors(tmp_path):
    txt = ("%%MatrixMarket matrix coordinate pattern general\n"
           "% comment\n"
           "3 4 3\n"
           "1 2\n3 4\n2 1\n")
    (tmp_path / "p.mtx").write_text(txt)
    D = fileio.read_mtx(str(tmp_path / "p.mtx")).toarray()
    want = np.zeros((3, 4)); want[0, 1] = want[2, 3] = want[1, 0] = 1
    assert np.array_equal(D, want)
    skew = ("%%MatrixMarket matrix coordinate real skew-symmetric\n"
            "3 3 2\n2 1 1.5\n3 1 -4e-1\n")
    (tmp_path / "z.mtx").write_text(skew)
    Z = fileio.read_mtx(str(tmp_path / "z.mtx")).toarray()
    assert np.array_equal(Z, np.array([[0, -1.5, 0.4], [1.5, 0, 0], [-0.4, 0, 0]]))
    (tmp_path / "d.mtx").write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(G.UnsupportedError):
        fileio.read_mtx(str(tmp_path / "d.mtx"))
    (tmp_path / "b.mtx").write_text("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n")
    with pytest.raises(G.ArgumentError):
        fileio.read_mtx(str(tmp_path / "b.mtx"))
    (tmp_path / "t.mtx").write_text("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n")
    with pytest.raises(G.ArgumentError):
        fileio.read_mtx(str(tmp_path / "t.mtx"))
