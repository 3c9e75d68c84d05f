"""The GPU Matrix Market / .dat conversion (dbd_read_csr_gpu) against the host
conversion (dbd_read_csr, byte-identical to the reference's make_CSR): the
same CSR and the same .csr cache bytes on general, symmetric, pattern and
.dat files with comments, CRLF line ends, lines long enough for fgets to
split, values in every form strtod reads, and a file large enough for many
text tiles and three radix passes; the same errors on malformed files."""
import os
import shutil

import numpy as np
import pytest

import dbd_gb300 as dbd

pytestmark = pytest.mark.gpu


def value_text(rng):
    r = rng.random()
    if r < 0.5:
        return f"{rng.standard_normal() * 10.0 ** int(rng.integers(-5, 6)):.{int(rng.integers(1, 18))}g}"
    if r < 0.7:
        return str(int(rng.integers(-1000, 1000)))
    if r < 0.8:
        digits = "".join(rng.choice(list("0123456789"), int(rng.integers(18, 60))))
        return digits[:3] + "." + digits[3:] + f"e{int(rng.integers(-330, 310))}"
    return str(rng.choice(["0x1.8p3", "-0x.4p-2", "inf", "-inf", "nan", "1e-320", "3.4028236e38", "7e-46",
                           "1.5\r", "2.5e", "+0.5", "-0", ".25", "5."]))


def write_mm(path, nr, nc, entries, symmetric=False, header=True, comments=True, crlf=False, pattern=False):
    end = "\r\n" if crlf else "\n"
    with open(path, "w", newline="") as f:
        if header:
            f.write(f"%%MatrixMarket matrix coordinate {'pattern' if pattern else 'real'} "
                    f"{'symmetric' if symmetric else 'general'}{end}")
        if comments:
            f.write(f"% a comment{end}% another, with, commas{end}")
        f.write(f"{nr} {nc} {len(entries)}{end}")
        for e in entries:
            f.write(e + end)


def entries(rng, n, nr, nc, pattern=False, symmetric=False):
    out = []
    for _ in range(n):
        i, j = int(rng.integers(1, nr + 1)), int(rng.integers(1, nc + 1))
        if symmetric and j > i:
            i, j = j, i
        sep = str(rng.choice([" ", "\t", ",", "  ", " ,\t"]))
        out.append(f"{i}{sep}{j}" if pattern else f"{i}{sep}{j}{sep}{value_text(rng)}")
    return out


def both(tmp_path, name, writer):
    """Writes the file twice (host and GPU directories) and converts both."""
    res = {}
    for side in ("host", "gpu"):
        d = tmp_path / side
        d.mkdir(exist_ok=True)
        writer(str(d / name))
        res[side] = dbd.read_CSR(str(d / name), gpu=0 if side == "gpu" else None)
    return res, (tmp_path / "host" / (name + ".csr")).read_bytes(), (tmp_path / "gpu" / (name + ".csr")).read_bytes()


def same(res, cache_h, cache_g):
    h, g = res["host"], res["gpu"]
    assert (h.n_rows, h.n_cols, h.nnz) == (g.n_rows, g.n_cols, g.nnz)
    assert np.array_equal(h.row_ptr, g.row_ptr) and np.array_equal(h.col_idx, g.col_idx)
    assert np.array_equal(h.val.view(np.uint64), g.val.view(np.uint64))
    assert cache_h == cache_g


@pytest.mark.parametrize("kind", ["general", "symmetric", "pattern", "crlf"])
def test_small_files_match_host_conversion(tmp_path, kind):
    rng = np.random.default_rng(["general", "symmetric", "pattern", "crlf"].index(kind))
    nr, nc = 300, 250
    sym = kind == "symmetric"
    ents = entries(rng, 4000, nr, nr if sym else nc, pattern=kind == "pattern", symmetric=sym)
    res, ch, cg = both(tmp_path, "m.mtx", lambda p: write_mm(p, nr, nr if sym else nc, ents, symmetric=sym,
                                                          crlf=kind == "crlf", pattern=kind == "pattern"))
    same(res, ch, cg)
    assert res["gpu"].nnz >= 4000


def test_dat_file_and_long_lines(tmp_path):
    rng = np.random.default_rng(7)
    ents = entries(rng, 500, 40, 40)
    # A line of 206 characters: fgets reads it as two pieces, each an entry.
    ents.insert(10, ("3 4 2.5" + " " * 192)[:199] + "5 6 7.5")
    ents.insert(20, "8 9")  # no value: 1.0
    ents.insert(30, "10 11 ")  # a trailing delimiter: the newline is the third token, read as 0.0

    def w(p):
        with open(p, "w") as f:
            f.write(f"40 40 {len(ents)}\n")
            for e in ents:
                f.write(e + "\n")
            f.write("   \t ")  # a last piece without tokens
    res, ch, cg = both(tmp_path, "m.dat", w)
    same(res, ch, cg)
    assert res["gpu"].nnz == len(ents) + 1


def test_large_file_many_tiles_and_radix_passes(tmp_path):
    rng = np.random.default_rng(9)
    nr = nc = 150000  # 18 bits of row index: three radix passes
    n = 600000
    i = rng.integers(1, nr + 1, n)
    j = rng.integers(1, nc + 1, n)
    v = rng.standard_normal(n)

    def w(p):
        with open(p, "w") as f:
            f.write("%%MatrixMarket matrix coordinate real general\n")
            f.write(f"{nr} {nc} {n}\n")
            f.write("".join(f"{a} {b} {x:.17g}\n" for a, b, x in zip(i, j, v)))
    res, ch, cg = both(tmp_path, "big.mtx", w)
    same(res, ch, cg)
    # Stable by row: within a row the entries keep the file's order.
    g = res["gpu"]
    r = 77
    order = np.nonzero(i == r)[0]
    assert np.array_equal(g.col_idx[g.row_ptr[r]:g.row_ptr[r + 1]], j[order])


def test_empty_body(tmp_path):
    res, ch, cg = both(tmp_path, "e.mtx", lambda p: write_mm(p, 5, 5, []))
    same(res, ch, cg)
    assert res["gpu"].nnz == 0


@pytest.mark.parametrize("bad", ["single token", "outside"])
def test_errors_match(tmp_path, bad):
    ents = ["1 1 1.0", "2 2 2.0", "3" if bad == "single token" else "9 2 1.0", "3 3 3.0"]
    for side in ("host", "gpu"):
        d = tmp_path / side
        d.mkdir()
        write_mm(str(d / "x.mtx"), 4, 4, ents, comments=False)
        with pytest.raises(dbd.DBDError) as e:
            dbd.read_CSR(str(d / "x.mtx"), gpu=0 if side == "gpu" else None)
        assert e.value.code == -5  # DBD_ERR_IO
        assert not (d / "x.mtx.csr").exists()
