"""TEST INFRASTRUCTURE: numpy restatement of the checkpoint record.

Only tests/ use this module, as the checker of les_fortran_record_* and
les_checkpoint_*.

Record format: the unformatted sequential layout of gfortran and Intel
Fortran with 4-byte markers (the reference is built with ifort,
compile.sh:7, and writes its checkpoint with a plain `write (lun)`,
io.f90:1325-1335).  A logical record is one or more subrecords; each is a
leading marker, at most 2147483639 data bytes and a trailing marker.  A
marker holds the subrecord's data length; the leading marker is negated
when another subrecord follows, the trailing marker when one precedes.
Little-endian throughout.

Parity unpinned: the reference ships no record file and no Fortran compiler
is available here, so this restatement follows the published description
of the format, not bytes the reference wrote.

Checkpoint layout: io.f90:1314-1338 (`checkpoint`), read back by
initial.f90:54-114 (with scalars, model 5, not inilag) and :128-160
(without scalars).  Array shapes: sim_param.f90:18-38 (ld,ny,lbz:nz),
scalars_module.f90:35-36, scalars_module_q.f90:21-22, bottombc.f90:17
(nx,ny), sgsmodule.f90:8-32 (ld,ny,nz).
"""
import numpy as np

MAX_SUB = 2147483639


def write_record(data, max_sub=MAX_SUB):
    """Bytes of one logical record holding the bytes `data`."""
    data = bytes(data)
    n = len(data)
    out = bytearray()
    pos, k = 0, 0
    while True:
        ln = min(max_sub, n - pos)
        more = n - pos > ln
        out += np.int32(-ln if more else ln).astype("<i4").tobytes()
        out += data[pos:pos + ln]
        out += np.int32(-ln if k > 0 else ln).astype("<i4").tobytes()
        pos += ln
        k += 1
        if not more:
            return bytes(out)


def read_record(buf, offset=0):
    """(data bytes, offset of the next record) of the record at offset."""
    data = bytearray()
    k = 0
    while True:
        head = int(np.frombuffer(buf, "<i4", 1, offset)[0])
        ln = abs(head)
        data += buf[offset + 4:offset + 4 + ln]
        tail = int(np.frombuffer(buf, "<i4", 1, offset + 4 + ln)[0])
        if abs(tail) != ln or (tail < 0) != (k > 0):
            raise ValueError("record markers do not match")
        offset += ln + 8
        k += 1
        if head >= 0:
            return bytes(data), offset


def checkpoint_items(nx, ny, nz, s_flag):
    """(name, shape) of the checkpoint record in order; shapes are Fortran
    (column-major) shapes of the arrays as written."""
    ld = nx + 2
    vol = (ld, ny, nz)
    if s_flag:
        names = [("u", vol), ("v", vol), ("w", vol), ("theta", vol), ("qmix", vol),
                 ("RHSx", vol), ("RHSy", vol), ("RHSz", vol), ("RHS_T", vol), ("RHS_q", vol),
                 ("sgs_t3", (ld, ny)), ("sgs_q3", (ld, ny)),
                 ("psi_m", (nx, ny)), ("psi_m0", (nx, ny)), ("psi_h", (nx, ny)), ("psi_h0", (nx, ny)),
                 ("Cs_opt2", vol), ("F_LM", vol), ("F_MM", vol), ("F_QN", vol), ("F_NN", vol),
                 ("G_LM", vol), ("G_MM", vol), ("G_QN", vol), ("G_NN", vol), ("Pr_t", vol)]
    else:
        names = [("u", vol), ("v", vol), ("w", vol), ("RHSx", vol), ("RHSy", vol), ("RHSz", vol),
                 ("Cs_opt2", vol), ("F_LM", vol), ("F_MM", vol), ("F_QN", vol), ("F_NN", vol)]
    return names


def split_checkpoint(data, nx, ny, nz, s_flag):
    """Arrays of a checkpoint record's data bytes, by name (Fortran order)."""
    out, pos = {}, 0
    for name, shape in checkpoint_items(nx, ny, nz, s_flag):
        n = int(np.prod(shape))
        out[name] = np.frombuffer(data, "<f8", n, pos).reshape(shape, order="F")
        pos += 8 * n
    if pos != len(data):
        raise ValueError("record holds %d bytes, the checkpoint list %d" % (len(data), pos))
    return out
