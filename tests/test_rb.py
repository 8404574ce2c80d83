"""Rutherford-Boeing reader/writer (host side)."""
import numpy as np

from spral_gb300 import matrices as M, rb


def test_rb_roundtrip(tmp_path):
    p, r, v = M.laplacian_2d(7, 5, -0.3)
    v = v * np.random.default_rng(0).uniform(0.5, 1.5, v.size)
    f = tmp_path / "lap.rb"
    rb.rb_write(str(f), p, r, v, "rsa", title="shifted Laplacian", identifier="lap75")
    m, n, p2, r2, v2, tc = rb.rb_read(str(f))
    assert (m, n, tc) == (35, 35, "rsa")
    assert np.array_equal(p2, p) and np.array_equal(r2, r)
    assert np.array_equal(v2, v)  # 17 significant digits round-trip exactly


def test_rb_reads_fortran_formats_and_patterns(tmp_path):
    # a 3x3 symmetric matrix in Fortran D-exponent format, hand written
    text = (
        f"{'tiny test matrix':<72}{'tiny':<8}\n"
        f"{5:14d}{1:14d}{1:14d}{2:14d}\n"
        f"{'rsa':<3}{'':11}{3:14d}{3:14d}{5:14d}{0:14d}\n"
        f"{'(4I5)':<16}{'(5I5)':<16}{'(1P,3D25.16)':<20}\n"
        "    1    4    5    6\n"
        "    1    2    3    2    3\n"
        "   4.0000000000000000D+00  -1.0000000000000000D+00   5.0000000000000000D-01\n"
        "   3.0000000000000000D+00   2.0000000000000000D+00\n")
    f = tmp_path / "tiny.rb"
    f.write_text(text)
    m, n, p, r, v, tc = rb.rb_read(str(f))
    assert (m, n) == (3, 3)
    assert p.tolist() == [0, 3, 4, 5] and r.tolist() == [0, 1, 2, 1, 2]
    assert v.tolist() == [4.0, -1.0, 0.5, 3.0, 2.0]
    # pattern only: values are made up; "dominant" gives an SPD matrix
    pat = text.replace("rsa", "psa").rsplit("   4.0", 1)[0]
    f2 = tmp_path / "pat.rb"
    f2.write_text(pat)
    *_, vd, tc2 = rb.rb_read(str(f2), make_values="dominant")
    assert tc2 == "psa"
    A = np.zeros((3, 3))
    for j in range(3):
        for k in range(p[j], p[j + 1]):
            A[r[k], j] = A[j, r[k]] = vd[k]
    assert np.all(np.linalg.eigvalsh(A) > 0)
