"""The extraction-file oracle (XTR version 5) against the header bytes HemeLB's own
test expects, and its distribution-checkpoint layout (no GPU)."""
import json
import struct
from pathlib import Path

import numpy as np
import pytest

from oracle import xtr as X

GOLDEN = json.loads((Path(__file__).parent / "golden" / "xtr_header.json").read_text())


def test_stored_string_lengths_match_reference():
    for s, n in GOLDEN["stored_string_lengths"].items():
        assert X.stored_length_of_string(s) == n


def test_main_and_field_headers_match_reference_bytes():
    fh = [X.field_header(f["name"], f["nvalues"], f["type"], f["offsets"]) for f in GOLDEN["fields"]]
    assert b"".join(fh) == bytes.fromhex(GOLDEN["field_header_hex"])
    mh = X.main_header(GOLDEN["voxel_size"], GOLDEN["origin"], GOLDEN["site_count"], fh)
    assert mh == bytes.fromhex(GOLDEN["main_header_hex"])


def test_distribution_checkpoint_layout():
    """One field "distributions": 19 DOUBLE values, no offsets (a 32-byte field
    header), and per site 12 + 152 bytes after the uint64 timestep."""
    h = X.checkpoint_header(5, 0.3e-3, (0.034, 0.001, 0.074))
    assert len(h) == 60 + 32
    # everything up to the site count is the reference test's main header
    assert h[:44] == bytes.fromhex(GOLDEN["main_header_hex"])[:44]
    assert struct.unpack(">QII", h[44:60]) == (5, 1, 32)
    assert h[60:] == X.xdr_string("distributions") + struct.pack(">III", 19, 1, 0)
    rng = np.random.default_rng(0)
    coords = rng.integers(0, 1000, (5, 3))
    f = rng.standard_normal((5, 19))
    rec = X.checkpoint_record(42, coords, f)
    assert len(rec) == 8 + 5 * (12 + 152)
    hdr, recs = X.read_checkpoint(h + rec + X.checkpoint_record(43, coords, 2 * f))
    assert hdr["site_count"] == 5 and hdr["voxel_size"] == 0.3e-3
    assert [r[0] for r in recs] == [42, 43]
    assert np.array_equal(recs[0][1], coords) and np.array_equal(recs[0][2], f)
    assert X.select_record(recs)[0] == 43 and X.select_record(recs, 42)[0] == 42
    with pytest.raises(ValueError):
        X.select_record(recs, 44)
    with pytest.raises(ValueError):
        X.read_checkpoint(h + rec[:-8])
    bad = bytearray(h + rec)
    bad[11] = 4  # version 4
    with pytest.raises(ValueError):
        X.read_checkpoint(bytes(bad))


def test_offset_file_of_one_writer():
    off = X.offset_file(92, 8 + 5 * 164)
    assert struct.unpack(">IIIi", off[:16]) == (0x686C6221, 0x6F666604, 1, 1)
    assert struct.unpack(">QQ", off[16:]) == (92, 92 + 8 + 5 * 164)
