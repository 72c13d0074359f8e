"""Writes xtr_header.json: the extraction-file (XTR version 5) header bytes that
HemeLB's own test expects (Code/tests/extraction/LocalPropertyOutputTests.cc, the
"Write" section: expectedMainHeader and expectedFieldHeader) together with the
inputs they were written from (Code/tests/extraction/DummyDataSource.h: 64 sites,
voxel size 0.3e-3, origin (0.034, 0.001, 0.074); fields "Pressure", one FLOAT
value with the offset 8.0 (REFERENCE_PRESSURE_mmHg), and "Velocity", three FLOAT
values without offsets).  The byte strings are read from the test's C string
literals, so the fixture is the reference's own golden vector.

Run from the repository root with the reference checkout as the argument:
    python tests/golden/make_xtr_golden.py <hemelb checkout>
"""
import json
import re
import sys
from pathlib import Path


def c_literal_bytes(src: str, name: str) -> bytes:
    """The concatenated string literals of `const char name[] = "..." "...";`."""
    m = re.search(r"const char " + name + r"\[\]\s*=(.*?);", src, re.S)
    body = re.sub(r"//[^\n]*", "", m.group(1))
    out = bytearray()
    for lit in re.findall(r'"((?:[^"\\]|\\.)*)"', body):
        i = 0
        while i < len(lit):
            if lit[i] == "\\" and lit[i + 1] == "x":
                out.append(int(lit[i + 2:i + 4], 16))
                i += 4
            else:
                out.append(ord(lit[i]))
                i += 1
    return bytes(out)


def main(ref: Path):
    src = (ref / "Code/tests/extraction/LocalPropertyOutputTests.cc").read_text()
    main_h = c_literal_bytes(src, "expectedMainHeader")
    field_h = c_literal_bytes(src, "expectedFieldHeader")
    assert len(main_h) == 60 and len(field_h) == 0x34
    out = {
        "source": "Code/tests/extraction/LocalPropertyOutputTests.cc (Write section)",
        "voxel_size": 0.3e-3,
        "origin": [0.034, 0.001, 0.074],
        "site_count": 64,
        "fields": [
            {"name": "Pressure", "nvalues": 1, "type": "FLOAT", "offsets": [8.0]},
            {"name": "Velocity", "nvalues": 3, "type": "FLOAT", "offsets": []},
        ],
        "main_header_hex": main_h.hex(),
        "field_header_hex": field_h.hex(),
        "stored_string_lengths": {"": 4, "Fish": 8, "A": 8},
    }
    Path(__file__).with_name("xtr_header.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main(Path(sys.argv[1]))
