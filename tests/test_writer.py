"""The +I/O output writer (dbd_writer_*) on the host, no GPU: aligned
O_DIRECT appends of ragged chunks, the reference's float32/int32 layout, and
its failure paths made on the host -- a disk that is full (/dev/full and an
injected ENOSPC), short writes, a stalled disk, an interrupted run resumed
from its progress manifest.  DBD_IO_FAULT is the writer's host-side fault
injection (enospc@N, short@N, stall@MS)."""
import os
import shutil

import numpy as np
import pytest

import dbd_gb300 as dbd


def product(m, seed, max_row=3000):
    rng = np.random.default_rng(seed)
    cnt = rng.integers(0, max_row, m)
    cnt[rng.random(m) < 0.2] = 0
    ptr = np.zeros(m + 1, np.int64)
    np.cumsum(cnt, out=ptr[1:])
    idx = rng.integers(0, 1 << 30, int(ptr[-1])).astype(np.int32)
    val = rng.standard_normal(int(ptr[-1]))
    return ptr, idx, val


def chunks(ptr, seed):
    """Row boundaries of ragged chunks (some empty, some of one row)."""
    rng = np.random.default_rng(seed)
    m = ptr.size - 1
    cuts = np.unique(np.concatenate([[0, m], rng.integers(0, m + 1, 12)]))
    return list(zip(cuts[:-1], cuts[1:]))


def write_all(out, ptr, idx, val, seed=0, start_row=0, **kw):
    w = dbd.Writer(str(out), ptr.size - 1, int(ptr[-1]), **kw)
    for r0, r1 in chunks(ptr, seed):
        if r1 <= start_row:
            continue
        e0, e1 = ptr[r0], ptr[r1]
        w.append(r1, idx[e0:e1], val[e0:e1])
    t = w.finish(ptr)
    direct = w.direct
    w.close()
    return t, direct


def read_back(out, fp32=False, ptr32=False):
    return (np.fromfile(out / "Ptr.output", np.int32 if ptr32 else np.int64),
            np.fromfile(out / "Idx.output", np.int32),
            np.fromfile(out / "Val.output", np.float32 if fp32 else np.float64))


@pytest.mark.parametrize("buffered", [False, True])
def test_ragged_chunks_round_trip(tmp_path, buffered):
    ptr, idx, val = product(700, 1)
    _, direct = write_all(tmp_path, ptr, idx, val, buffered=buffered)
    if buffered:
        assert not direct
    p, i, v = read_back(tmp_path)
    assert np.array_equal(p, ptr) and np.array_equal(i, idx) and np.array_equal(v, val)
    assert os.path.getsize(tmp_path / "Idx.output") == 4 * ptr[-1]  # the padded tail block was cut


def test_reference_layout(tmp_path):
    ptr, idx, val = product(300, 2)
    write_all(tmp_path, ptr, idx, val, val_fp32=True, ptr32=True)
    p, i, v = read_back(tmp_path, fp32=True, ptr32=True)
    assert np.array_equal(p, ptr.astype(np.int32)) and np.array_equal(i, idx)
    assert np.array_equal(v, val.astype(np.float32))


def test_ptr32_overflow_is_refused(tmp_path):
    w = dbd.Writer(str(tmp_path), 1, 1 << 31, ptr32=True, buffered=True)
    with pytest.raises(dbd.DBDError) as e:
        w.finish(np.array([0, 1 << 31], np.int64))
    assert e.value.code == -8  # DBD_ERR_OVERFLOW
    w.close()


def test_full_disk_dev_full(tmp_path):
    """Idx.output pre-created as a link to /dev/full: ENOSPC, reported as DBD_ERR_IO."""
    if not os.path.exists("/dev/full"):
        pytest.skip("no /dev/full")
    os.symlink("/dev/full", tmp_path / "Idx.output")
    ptr, idx, val = product(200, 3)
    with pytest.raises(dbd.DBDError) as e:
        write_all(tmp_path, ptr, idx, val)
    assert e.value.code == -5 and "No space left" in str(e.value)


@pytest.mark.parametrize("buffered", [False, True])
def test_injected_enospc(tmp_path, monkeypatch, buffered):
    monkeypatch.setenv("DBD_IO_FAULT", "enospc@100000")
    ptr, idx, val = product(400, 4)
    with pytest.raises(dbd.DBDError) as e:
        write_all(tmp_path, ptr, idx, val, buffered=buffered)
    assert e.value.code == -5 and "No space left" in str(e.value)


@pytest.mark.parametrize("buffered", [False, True])
def test_short_writes_are_continued(tmp_path, monkeypatch, buffered):
    monkeypatch.setenv("DBD_IO_FAULT", "short@50000")
    ptr, idx, val = product(400, 5)
    write_all(tmp_path, ptr, idx, val, buffered=buffered)
    p, i, v = read_back(tmp_path)
    assert np.array_equal(p, ptr) and np.array_equal(i, idx) and np.array_equal(v, val)


def test_stalled_disk_completes(tmp_path, monkeypatch):
    monkeypatch.setenv("DBD_IO_FAULT", "stall@20")
    ptr, idx, val = product(60, 6, max_row=100)
    write_all(tmp_path, ptr, idx, val)
    p, i, v = read_back(tmp_path)
    assert np.array_equal(i, idx) and np.array_equal(v, val)


@pytest.mark.parametrize("buffered", [False, True])
def test_interrupted_run_resumes(tmp_path, monkeypatch, buffered):
    """A run dies of ENOSPC part way; the next run on the same product picks
    up after the last durable chunk and the files come out whole."""
    ptr, idx, val = product(900, 7)
    fp = 0x1234
    monkeypatch.setenv("DBD_IO_FAULT", f"enospc@{int(6 * ptr[-1])}")  # about half of the bytes
    with pytest.raises(dbd.DBDError):
        write_all(tmp_path, ptr, idx, val, resume=True, fingerprint=fp, buffered=buffered)
    assert (tmp_path / "DBD.progress").exists()
    monkeypatch.delenv("DBD_IO_FAULT")
    # Another product's run (a copy of the files, another fingerprint) starts afresh.
    shutil.copytree(tmp_path, tmp_path.parent / (tmp_path.name + "_other"))
    w = dbd.Writer(str(tmp_path.parent / (tmp_path.name + "_other")), 900, int(ptr[-1]), fingerprint=fp + 1,
                   resume=True, buffered=buffered)
    assert w.resume_row == 0
    w.close()
    w = dbd.Writer(str(tmp_path), 900, int(ptr[-1]), fingerprint=fp, resume=True, buffered=buffered)
    start = w.resume_row
    w.close()
    assert 0 < start < 900
    assert start in {r1 for _, r1 in chunks(ptr, 0)}
    write_all(tmp_path, ptr, idx, val, start_row=start, resume=True, fingerprint=fp, buffered=buffered)
    p, i, v = read_back(tmp_path)
    assert np.array_equal(p, ptr) and np.array_equal(i, idx) and np.array_equal(v, val)
    assert not (tmp_path / "DBD.progress").exists()


def test_resume_and_rotation_exclusive(tmp_path):
    with pytest.raises(dbd.DBDError):
        dbd.Writer(str(tmp_path), 10, 10, resume=True, rotate_gib=1.0)
