"""Record layer of the checkpoint (les_fortran_record_write / _read, host
only, no GPU) against the numpy restatement of the Fortran unformatted
sequential format in oracle/fortran_record.py: byte-identical records,
subrecord splitting, prefix reads and the errors a damaged file raises."""
import os

import numpy as np
import pytest

from oracle import fortran_record as fr


def _data(n, seed):
    return np.random.default_rng(seed).integers(0, 256, n, dtype=np.uint8)


@pytest.mark.parametrize("n,max_sub", [(0, 0), (1, 0), (800, 0), (800, 8), (800, 100), (800, 799),
                                       (801, 267), (8 * 1000 + 5, 1000)])
def test_writer_matches_restatement(gpu_lib, tmp_path, n, max_sub):
    d = _data(n, n + max_sub)
    p = str(tmp_path / "r.bin")
    # the data in three parts, cut at arbitrary points
    cuts = [0, n // 3, (2 * n) // 3, n]
    gpu_lib.fortran_record_write(p, [d[cuts[i]:cuts[i + 1]] for i in range(3)], max_subrecord=max_sub)
    ref = fr.write_record(d.tobytes(), max_sub if max_sub > 0 else fr.MAX_SUB)
    assert open(p, "rb").read() == ref
    back, nxt = fr.read_record(ref)
    assert back == d.tobytes() and nxt == len(ref)


def test_reader_walks_appended_records(gpu_lib, tmp_path):
    recs = [_data(n, n) for n in (40, 0, 333, 1000)]
    buf = b"".join(fr.write_record(r.tobytes(), 64) for r in recs)
    p = str(tmp_path / "m.bin")
    open(p, "wb").write(buf)
    off = 0
    for r in recs:
        bufs, ln, nxt = gpu_lib.fortran_record_read(p, [len(r)], offset=off)
        assert ln == len(r) and np.array_equal(bufs[0], r)
        off = nxt
    assert off == len(buf)


def test_prefix_read_skips_the_rest(gpu_lib, tmp_path):
    # a Fortran read of a shorter list takes the front of the record
    d = _data(1000, 7)
    p = str(tmp_path / "p.bin")
    open(p, "wb").write(fr.write_record(d.tobytes(), 300) + fr.write_record(b"tail", 300))
    bufs, ln, nxt = gpu_lib.fortran_record_read(p, [10, 500])
    assert ln == 1000 and bytes(bufs[0]) + bytes(bufs[1]) == d[:510].tobytes()
    bufs, ln, _ = gpu_lib.fortran_record_read(p, [4], offset=nxt)
    assert bytes(bufs[0]) == b"tail"


def test_length_only_read(gpu_lib, tmp_path):
    # no buffers: the record's length and the next offset (how the checkpoint
    # reader checks a file before changing any field)
    p = str(tmp_path / "l.bin")
    open(p, "wb").write(fr.write_record(b"x" * 700, 256) + fr.write_record(b"yz", 256))
    bufs, ln, nxt = gpu_lib.fortran_record_read(p, [])
    assert bufs == [] and ln == 700 and nxt == 700 + 3 * 8
    _, ln2, nxt2 = gpu_lib.fortran_record_read(p, [], offset=nxt)
    assert ln2 == 2 and nxt2 == 700 + 3 * 8 + 2 + 8


def test_appending_writer(gpu_lib, tmp_path):
    p = str(tmp_path / "a.bin")
    a, b = _data(100, 1), _data(50, 2)
    gpu_lib.fortran_record_write(p, [a], max_subrecord=30)
    gpu_lib.fortran_record_write(p, [b], append=True, max_subrecord=30)
    assert open(p, "rb").read() == fr.write_record(a.tobytes(), 30) + fr.write_record(b.tobytes(), 30)


@pytest.mark.parametrize("damage", ["short_list", "truncated", "tail_marker", "continuation_sign", "no_record"])
def test_damaged_records_raise(gpu_lib, tmp_path, damage):
    d = _data(600, 3)
    raw = bytearray(fr.write_record(d.tobytes(), 256))
    want = [600]
    if damage == "short_list":
        want = [601]
    elif damage == "truncated":
        raw = raw[:-10]
    elif damage == "tail_marker":
        raw[4 + 256:4 + 256 + 4] = np.int32(255).astype("<i4").tobytes()
    elif damage == "continuation_sign":  # second subrecord's trailing marker not negated
        off = 4 + 256 + 4
        raw[off + 4 + 256:off + 4 + 256 + 4] = np.int32(256).astype("<i4").tobytes()
    p = str(tmp_path / "d.bin")
    open(p, "wb").write(bytes(raw))
    off = len(raw) if damage == "no_record" else 0
    with pytest.raises(gpu_lib.LesError) as e:
        gpu_lib.fortran_record_read(p, want, offset=off)
    assert e.value.code == -10


def test_checkpoint_layout_sizes():
    # io.f90:1325-1335: 20 (ld,ny,nz) arrays, two (ld,ny) and four (nx,ny)
    # planes with scalars; 11 (ld,ny,nz) arrays without
    nx, ny, nz = 32, 32, 33
    ld = nx + 2
    s1 = sum(int(np.prod(s)) for _, s in fr.checkpoint_items(nx, ny, nz, 1))
    s0 = sum(int(np.prod(s)) for _, s in fr.checkpoint_items(nx, ny, nz, 0))
    assert s1 == 20 * ld * ny * nz + 2 * ld * ny + 4 * nx * ny
    assert s0 == 11 * ld * ny * nz
    # a 256^3 record with scalars needs two subrecords
    assert 8 * (20 * 258 * 256 * 257 + 2 * 258 * 256 + 4 * 256 * 256) > fr.MAX_SUB
