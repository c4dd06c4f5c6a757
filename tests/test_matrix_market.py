"""MatrixMarket input and the driver's setup around it (include/senk_io.hpp,
senk::matrix::Expand / GetDiag / Scaling) against the oracle and, where the
reference sources are present, the reference itself. Files are written from
the synthetic systems: general and symmetric, with comment lines, explicit
zeros, scientific notation and shuffled entry order."""
import numpy as np
import pytest

from senk_gb300 import problems as P
from senk_gb300 import setup as S


def _write(path, A, symmetric=False, zeros=0, seed=0, comments=2, fmt="%.17g", header=None):
    rng = np.random.default_rng(seed)
    rows = np.repeat(np.arange(A.n), np.diff(A.rptr))
    cols = A.cind.astype(np.int64)
    vals = A.val.astype(np.float64)
    if symmetric:
        keep = cols <= rows
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
    if zeros:
        # explicit zero entries at free positions of the lower triangle
        zr = rng.integers(1, A.n, zeros)
        zc = np.maximum(zr - 2 - rng.integers(0, 3, zeros), 0)
        taken = set(zip(rows.tolist(), cols.tolist()))
        extra = [(r, c) for r, c in zip(zr.tolist(), zc.tolist()) if (r, c) not in taken]
        extra = list(dict.fromkeys(extra))
        if extra:
            er, ec = np.array(extra).T
            rows = np.concatenate([rows, er])
            cols = np.concatenate([cols, ec])
            vals = np.concatenate([vals, np.zeros(len(extra))])
    order = rng.permutation(len(rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    with open(path, "w") as f:
        f.write(header or ("%%MatrixMarket matrix coordinate real " + ("symmetric" if symmetric else "general") + "\n"))
        for k in range(comments):
            f.write(f"% comment line {k}\n")
        f.write(f"{A.n} {A.n} {len(rows)}\n")
        for r, c, v in zip(rows, cols, vals):
            f.write(f"{r + 1} {c + 1} {fmt % v}\n")
    return len(rows)


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes()


CASES = {
    "poisson32": lambda: P.poisson2d(32),
    "convdiff10": lambda: P.convdiff3d(10, 0.5),
    "vardiff8": lambda: P.vardiff3d(8, 1.5, 4.0, 3),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("remove_zeros", [True, False])
def test_reader_matches_oracle(tmp_path, port, case, symmetric, remove_zeros):
    A = CASES[case]()
    path = tmp_path / "a.mtx"
    _write(path, A, symmetric, zeros=7, seed=len(case))
    B, M, sym = S.ReadMatrixMarket(path, remove_zeros)
    o = port.read_matrix_market(path, remove_zeros)
    assert o is not None
    ov, oc, orp, on, om, osym = o
    assert sym == osym == symmetric and B.n == on == A.n and M == om == A.n
    assert _same(B.rptr, orp) and _same(B.cind, oc) and _same(B.val, ov)
    if not symmetric and remove_zeros:
        # the file held A plus explicit zeros: reading drops them and sorts the rows
        assert _same(B.rptr, A.rptr) and _same(B.cind, A.cind.astype(np.int32)) and _same(B.val, A.val)


@pytest.mark.parametrize("case", sorted(CASES))
def test_reader_and_expand_match_reference(tmp_path, port, ref, case):
    A = CASES[case]()
    for symmetric in (False, True):
        path = tmp_path / f"a{int(symmetric)}.mtx"
        _write(path, A, symmetric, zeros=5, seed=3, fmt="%.16e")
        B, M, sym = S.ReadMatrixMarket(path, True)
        r = ref.read_matrix_market(path, True)
        rv, rc, rrp, rn, rm, rsym = r
        assert sym == rsym and B.n == rn and M == rm
        assert _same(B.rptr, rrp) and _same(B.cind, rc) and _same(B.val, rv)
        text = ref.last_stdout.value.decode()
        assert "# Readfile MatrixMarket" in text and f"# {A.n} {A.n} " in text
        if symmetric:
            E, Eo, Er = S.Expand(B, "L"), port.expand(B, "L"), ref.expand(B, "L")
            for X in (Eo, Er):
                assert _same(E.rptr, X.rptr) and _same(E.cind, X.cind) and _same(E.val, X.val)
            # the full symmetric matrix the file came from (the synthetic systems
            # are not symmetric, so compare with the lower triangle mirrored)
            lo = (np.repeat(np.arange(A.n), np.diff(A.rptr)), A.cind)
            assert E.nnz == 2 * int(np.sum(lo[1] <= lo[0])) - A.n


def test_reader_large_file_parallel_chunks(tmp_path, port):
    # larger than one parse chunk per thread, so several threads join their parts
    A = P.convdiff3d(40, 0.5)
    path = tmp_path / "big.mtx"
    _write(path, A, False, zeros=50, seed=9)
    B, _, _ = S.ReadMatrixMarket(path, True)
    assert _same(B.rptr, A.rptr) and _same(B.cind, A.cind.astype(np.int32)) and _same(B.val, A.val)
    ov, oc, orp, *_ = port.read_matrix_market(path, True)
    assert _same(B.val, ov) and _same(B.cind, oc)


@pytest.mark.parametrize("bad", ["complex", "noshape", "short", "index", "token"])
def test_reader_rejects_bad_files(tmp_path, bad):
    A = P.poisson2d(8)
    path = tmp_path / "bad.mtx"
    if bad == "complex":
        _write(path, A, header="%%MatrixMarket matrix coordinate complex general\n")
    elif bad == "noshape":
        _write(path, A, header="%%MatrixMarket matrix coordinate real hermitian-ish\n")
    else:
        n = _write(path, A)
        lines = open(path).read().splitlines()
        if bad == "short":
            lines = lines[:-3]
        elif bad == "index":
            lines[-1] = f"{A.n + 5} 1 1.0"
        else:
            lines[5] = "3 x 1.0"
        open(path, "w").write("\n".join(lines) + "\n")
    with pytest.raises(S.SenkError):
        S.ReadMatrixMarket(path, True)


def test_extra_entries_beyond_the_size_line_are_ignored(tmp_path, port):
    A = P.poisson2d(8)
    path = tmp_path / "extra.mtx"
    _write(path, A, seed=1)
    with open(path, "a") as f:
        f.write("1 2 99.0\n3 3 7.0\n")
    B, _, _ = S.ReadMatrixMarket(path, True)
    assert _same(B.val, A.val) and _same(B.cind, A.cind.astype(np.int32))


def test_host_scaling_matches_reference(port, ref):
    A = P.vardiff3d(8, 1.5, 4.0, 3)
    d = port.get_diag(A)
    assert _same(d, ref.get_diag(A))
    inv = 1.0 / np.sqrt(np.abs(d))
    assert _same(port.scaling(A, inv, inv).val, ref.scaling(A, inv, inv).val)
