"""A reader of SDF files, the reference's dump format.

TEST INFRASTRUCTURE ONLY: the tests read the product's SDF output with it.
It restates the layout from the reference's SDF library sources (SDF/C
sdf_input.c and sdf.h for reading; SDF/FORTRAN sdf_output_ru.f90,
sdf_output_cartesian_ru.f90 and sdf_output_util.f90 for what is written):
a 112-byte header; blocks chained by next_block_location from
first_block_location, each a block header (next, data location, id,
data length, block type, data type, ndims, name, block-info length) with
type-specific metadata; and a summary at summary_location repeating every
block header and metadata.  Only the block types the product writes are
decoded (plain mesh 1, point mesh 2, plain variable 3, point variable 4,
constant 5; sdf_output_point_ru.f90 for the point types, sdf_output_ru.f90
write_constant_meta for constants: the value in the metadata, no data).
Parity status: unpinned -- the
reference's SDF reader needs a header its build generates and no SDF files
ship with the reference, so this restatement is the only reader here.
"""
import struct

import numpy as np

HEADER_LEN = 112


def _str(b):
    return b.split(b"\0", 1)[0].decode("ascii").rstrip(" ")


class Header:
    pass


def _header(buf):
    h = Header()
    h.magic = buf[0:4]
    (h.endianness, h.version, h.revision) = struct.unpack_from("<iii", buf, 4)
    h.code_name = _str(buf[16:48])
    (h.first_block_location, h.summary_location, h.summary_size, h.nblocks, h.block_header_length, h.step,
     h.time, h.jobid1, h.jobid2, h.string_length, h.code_io_version) = struct.unpack_from("<qqiiiidiiii", buf, 48)
    h.restart_flag, h.other_domains, h.station_file = buf[104], buf[105], buf[106]
    return h


def _block(buf, at, h):
    """The block header and metadata at offset `at`."""
    ids = 32
    sl = h.string_length
    b = {}
    b["start"] = at
    b["next_block_location"], b["data_location"] = struct.unpack_from("<qq", buf, at)
    b["id"] = _str(buf[at + 16:at + 16 + ids])
    o = at + 16 + ids
    b["data_length"], b["blocktype"], b["datatype"], b["ndims"] = struct.unpack_from("<qiii", buf, o)
    o += 20
    b["name"] = _str(buf[o:o + sl])
    o += sl
    (b["info_length"],) = struct.unpack_from("<i", buf, o)
    o += 4
    assert o - at == h.block_header_length
    nd = b["ndims"]
    if b["blocktype"] == 3:  # plain variable
        (b["mult"],) = struct.unpack_from("<d", buf, o)
        b["units"] = _str(buf[o + 8:o + 8 + ids])
        b["mesh_id"] = _str(buf[o + 8 + ids:o + 8 + 2 * ids])
        p = o + 8 + 2 * ids
        b["dims"] = list(struct.unpack_from("<" + "i" * nd, buf, p))
        (b["stagger"],) = struct.unpack_from("<i", buf, p + 4 * nd)
        meta = 8 + 2 * ids + 4 * nd + 4
    elif b["blocktype"] == 1:  # plain mesh
        b["mults"] = list(struct.unpack_from("<" + "d" * nd, buf, o))
        p = o + 8 * nd
        b["labels"] = [_str(buf[p + ids * i:p + ids * (i + 1)]) for i in range(nd)]
        p += ids * nd
        b["units"] = [_str(buf[p + ids * i:p + ids * (i + 1)]) for i in range(nd)]
        p += ids * nd
        (b["geometry"],) = struct.unpack_from("<i", buf, p)
        p += 4
        b["extents"] = list(struct.unpack_from("<" + "d" * (2 * nd), buf, p))
        p += 16 * nd
        b["dims"] = list(struct.unpack_from("<" + "i" * nd, buf, p))
        meta = 8 * nd + 2 * ids * nd + 4 + 16 * nd + 4 * nd
    elif b["blocktype"] == 2:  # point mesh
        b["mults"] = list(struct.unpack_from("<" + "d" * nd, buf, o))
        p = o + 8 * nd
        b["labels"] = [_str(buf[p + ids * i:p + ids * (i + 1)]) for i in range(nd)]
        p += ids * nd
        b["units"] = [_str(buf[p + ids * i:p + ids * (i + 1)]) for i in range(nd)]
        p += ids * nd
        (b["geometry"],) = struct.unpack_from("<i", buf, p)
        p += 4
        b["extents"] = list(struct.unpack_from("<" + "d" * (2 * nd), buf, p))
        p += 16 * nd
        (b["npoints"],) = struct.unpack_from("<q", buf, p)
        b["species_id"] = _str(buf[p + 8:p + 8 + ids])
        meta = 8 * nd + 2 * ids * nd + 4 + 16 * nd + 8 + ids
    elif b["blocktype"] == 4:  # point variable
        (b["mult"],) = struct.unpack_from("<d", buf, o)
        b["units"] = _str(buf[o + 8:o + 8 + ids])
        b["mesh_id"] = _str(buf[o + 8 + ids:o + 8 + 2 * ids])
        (b["npoints"],) = struct.unpack_from("<q", buf, o + 8 + 2 * ids)
        b["species_id"] = _str(buf[o + 16 + 2 * ids:o + 16 + 3 * ids])
        meta = 16 + 3 * ids
    elif b["blocktype"] == 5:  # constant
        fmt = {4: "<d", 2: "<q", 1: "<i"}[b["datatype"]]
        (b["value"],) = struct.unpack_from(fmt, buf, o)
        meta = struct.calcsize(fmt)
        assert b["data_length"] == 0
    else:
        meta = b["info_length"]
    assert b["info_length"] == meta, (b["id"], b["info_length"], meta)
    return b


def _data(buf, b):
    assert b["datatype"] in (2, 4), "integer8 and real8 only"
    dt = "<i8" if b["datatype"] == 2 else "<f8"
    a = np.frombuffer(buf, dtype=dt, count=b["data_length"] // 8, offset=b["data_location"])
    if b["blocktype"] == 2:
        return a.reshape(b["ndims"], b["npoints"]).copy()  # one row per dimension
    if b["blocktype"] == 4:
        return a.copy()
    if b["blocktype"] == 3:
        return a.reshape(b["dims"][::-1])  # Fortran order: (n_mode, ny, nx)
    if b["blocktype"] == 1:
        nx = b["dims"][0]
        return a[:nx].copy(), a[nx:].copy()
    return a


def read(path):
    """(header, inline blocks, summary blocks, {id: data}) of an SDF file."""
    with open(path, "rb") as f:
        buf = f.read()
    h = _header(buf)
    inline, at = [], h.first_block_location
    for _ in range(h.nblocks):
        b = _block(buf, at, h)
        inline.append(b)
        at = b["next_block_location"]
    summary, at = [], h.summary_location
    for _ in range(h.nblocks):
        b = _block(buf, at, h)
        summary.append(b)
        at = b["next_block_location"]
    data = {b["id"]: (b["value"] if b["blocktype"] == 5 else _data(buf, b)) for b in summary}
    h.file_size = len(buf)
    return h, inline, summary, data
