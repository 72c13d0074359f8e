"""CPU oracle of HemeLB's extraction files (XTR, version 5) as distribution
checkpoints (test infrastructure; only tests import this module).

Restates, in struct-packed Python:
  * the main header and field headers that LocalPropertyOutput::PrepareHeader
    writes (Code/extraction/LocalPropertyOutput.cc; constants in
    Code/io/formats/extraction.h: magic 0x78747204, version 5, 60-byte main
    header, XDR strings padded to 4 bytes after a 4-byte length),
  * one timestep record of a "distributions" field: the uint64 timestep, then per
    site its three uint32 grid coordinates and 19 doubles (LocalPropertyOutput::Write
    with LbDataSourceIterator::GetDistribution, which reads f_old),
  * the offset file of LocalPropertyOutput::WriteOffsetFile (Code/io/formats/offset.h:
    magic 0x6f666604, version 1, int32 rank count, rank count + 1 uint64 offsets),
  * and the reader's checks and timestep choice (LocalDistributionInput::LoadDistribution,
    Code/extraction/LocalDistributionInput.cc:56-251).
Pinned against the header bytes HemeLB's own test expects
(Code/tests/extraction/LocalPropertyOutputTests.cc; fixture tests/golden/xtr_header.json).
"""
from __future__ import annotations

import struct

import numpy as np

HEMELB_MAGIC = 0x686C6221
XTR_MAGIC = 0x78747204
XTR_VERSION = 5
OFF_MAGIC = 0x6F666604
OFF_VERSION = 1
TYPE_CODES = {"FLOAT": 0, "DOUBLE": 1, "INT32": 2, "UINT32": 3}
_OFFSET_FMT = {"FLOAT": ">f", "DOUBLE": ">d", "INT32": ">i", "UINT32": ">I"}


def xdr_string(s: str) -> bytes:
    b = s.encode()
    return struct.pack(">I", len(b)) + b + b"\0" * (-len(b) % 4)


def stored_length_of_string(s: str) -> int:
    return len(xdr_string(s))


def field_header(name: str, nvalues: int, type_name: str, offsets=()) -> bytes:
    h = xdr_string(name) + struct.pack(">III", nvalues, TYPE_CODES[type_name], len(offsets))
    return h + b"".join(struct.pack(_OFFSET_FMT[type_name], o) for o in offsets)


def main_header(voxel_size: float, origin, site_count: int, field_headers) -> bytes:
    fh = b"".join(field_headers)
    return (struct.pack(">III", HEMELB_MAGIC, XTR_MAGIC, XTR_VERSION) + struct.pack(">dddd", voxel_size, *origin)
            + struct.pack(">QII", site_count, len(field_headers), len(fh)))


def checkpoint_header(site_count: int, voxel_size: float = 1.0, origin=(0.0, 0.0, 0.0)) -> bytes:
    fh = field_header("distributions", 19, "DOUBLE")
    return main_header(voxel_size, origin, site_count, [fh]) + fh


def checkpoint_record(timestep: int, coords: np.ndarray, f: np.ndarray) -> bytes:
    """coords (n, 3) grid positions, f (n, 19) distributions, sites in file order."""
    n = coords.shape[0]
    rec = np.zeros(n, dtype=[("x", ">u4", 3), ("f", ">f8", 19)])
    rec["x"] = coords
    rec["f"] = f
    return struct.pack(">Q", timestep) + rec.tobytes()


def offset_file(header_len: int, record_len: int, ranks: int = 1) -> bytes:
    """Single-writer offsets: rank 0 holds the whole record, later ranks nothing."""
    offs = [header_len] + [header_len + record_len] * ranks
    return struct.pack(">IIIi", HEMELB_MAGIC, OFF_MAGIC, OFF_VERSION, ranks) + struct.pack(">%dQ" % len(offs), *offs)


def read_checkpoint(data: bytes):
    """Parse a distribution checkpoint: (header dict, [(timestep, coords, f), ...]).
    Raises ValueError where LocalDistributionInput would stop the run."""
    magic, xtr, ver = struct.unpack_from(">III", data, 0)
    if magic != HEMELB_MAGIC or xtr != XTR_MAGIC:
        raise ValueError("not an extraction file")
    if ver != XTR_VERSION:
        raise ValueError("extraction version is not 5")
    voxel, ox, oy, oz = struct.unpack_from(">dddd", data, 12)
    nsites, nfields, fhl = struct.unpack_from(">QII", data, 44)
    at = 60
    (ln,) = struct.unpack_from(">I", data, at)
    name = data[at + 4:at + 4 + ln].decode()
    at += 4 + ln + (-ln % 4)
    nelem, tcode, noff = struct.unpack_from(">III", data, at)
    at += 12
    if nfields != 1 or name != "distributions" or nelem != 19 or tcode != TYPE_CODES["DOUBLE"] or noff != 0 \
            or at - 60 != fhl:
        raise ValueError("not a D3Q19 distribution checkpoint")
    rec_len = 8 + nsites * (12 + 19 * 8)
    body = len(data) - at
    if body == 0 or body % rec_len:
        raise ValueError("length is not a whole number of timesteps")
    dt = np.dtype([("x", ">u4", 3), ("f", ">f8", 19)])
    records = []
    for k in range(body // rec_len):
        base = at + k * rec_len
        (ts,) = struct.unpack_from(">Q", data, base)
        rec = np.frombuffer(data, dtype=dt, count=nsites, offset=base + 8)
        records.append((ts, rec["x"].astype(np.int64), rec["f"].astype(np.float64)))
    header = {"voxel_size": voxel, "origin": (ox, oy, oz), "site_count": nsites}
    return header, records


def select_record(records, timestep: int = -1):
    """The record of `timestep`, or the last one when timestep < 0."""
    if timestep < 0:
        return records[-1]
    for r in records:
        if r[0] == timestep:
            return r
    raise ValueError("timestep not found")
