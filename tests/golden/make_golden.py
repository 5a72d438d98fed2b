"""Generate the golden fixtures of the parity tests from the reference tree.

Run it with the path of a checkout of the reference:

    python tests/golden/make_golden.py REFERENCE_ROOT

It reads, without executing anything from the reference:
  * python/test/data/standard_output_sum.tif              (uncompressed)
  * python/test/data/standard_output_sum_custom_shape.tif (LZW)
    -> decoded with the small baseline-TIFF reader below (TIFF 6.0 spec,
       sections 2 and 13) and saved as .npy
  * python/test/test_many.py -> the WKT list GEOMS and the burn values
    (`value` = 1..len(GEOMS)), saved as golden_inputs.json

The GPU machine has no reference tree; the tests only read the files written
here.
"""

from __future__ import annotations

import ast
import json
import struct
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _lzw_decode(data: bytes) -> bytes:
    """TIFF LZW (MSB-first codes, 9..12 bits, early change)."""
    CLEAR, EOI = 256, 257
    out = bytearray()
    table: list[bytes] = []

    def reset():
        nonlocal table
        table = [bytes([i]) for i in range(256)] + [b"", b""]

    reset()
    bitpos, nbits = 0, 9
    total = len(data) * 8
    prev = None
    while bitpos + nbits <= total:
        # read nbits MSB-first
        byte = bitpos >> 3
        chunk = int.from_bytes(data[byte:byte + 4].ljust(4, b"\0"), "big")
        code = (chunk >> (32 - (bitpos & 7) - nbits)) & ((1 << nbits) - 1)
        bitpos += nbits
        if code == EOI:
            break
        if code == CLEAR:
            reset()
            nbits = 9
            prev = None
            continue
        if prev is None:
            entry = table[code]
            out += entry
            prev = entry
            continue
        if code < len(table):
            entry = table[code]
            table.append(prev + entry[:1])
        else:
            entry = prev + prev[:1]
            table.append(entry)
        out += entry
        prev = entry
        if len(table) + 1 >= (1 << nbits) and nbits < 12:
            nbits += 1
    return bytes(out)


def read_tiff(path: Path) -> np.ndarray:
    raw = path.read_bytes()
    endian = {b"II": "<", b"MM": ">"}[raw[:2]]
    (magic,) = struct.unpack(endian + "H", raw[2:4])
    assert magic == 42, "BigTIFF not supported"
    (ifd,) = struct.unpack(endian + "I", raw[4:8])
    (n,) = struct.unpack(endian + "H", raw[ifd:ifd + 2])
    sizes = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 6: 1, 7: 1, 8: 2, 9: 4, 10: 8, 11: 4, 12: 8, 16: 8}
    fmts = {1: "B", 3: "H", 4: "I", 16: "Q", 6: "b", 8: "h", 9: "i"}
    tags = {}
    for k in range(n):
        e = raw[ifd + 2 + 12 * k: ifd + 14 + 12 * k]
        tag, typ, cnt = struct.unpack(endian + "HHI", e[:8])
        size = sizes[typ] * cnt
        body = e[8:12] if size <= 4 else raw[struct.unpack(endian + "I", e[8:12])[0]:][:size]
        if typ in fmts:
            tags[tag] = list(struct.unpack(endian + fmts[typ] * cnt, body[:size]))
    width, height = tags[256][0], tags[257][0]
    bps = tags.get(258, [1])[0]
    comp = tags.get(259, [1])[0]
    pred = tags.get(317, [1])[0]
    fmt = tags.get(339, [1])[0]
    offs, counts = tags[273], tags[279]
    buf = bytearray()
    for o, c in zip(offs, counts):
        strip = raw[o:o + c]
        if comp == 1:
            buf += strip
        elif comp == 5:
            buf += _lzw_decode(strip)
        else:
            raise ValueError(f"compression {comp} not supported")
    kind = {1: "u", 2: "i", 3: "f"}[fmt]
    dt = np.dtype(f"{endian}{kind}{bps // 8}")
    arr = np.frombuffer(bytes(buf[: width * height * dt.itemsize]), dtype=dt).reshape(height, width).copy()
    if pred == 2:
        arr = np.cumsum(arr, axis=1, dtype=arr.dtype)
    return arr.astype(dt.newbyteorder("="))


def read_geoms(test_file: Path) -> list[str]:
    tree = ast.parse(test_file.read_text())
    for node in tree.body:
        if isinstance(node, ast.Assign) and any(isinstance(t, ast.Name) and t.id == "GEOMS" for t in node.targets):
            return list(ast.literal_eval(node.value))
    raise ValueError("GEOMS not found")


def main(ref_root: Path) -> None:
    data = ref_root / "python" / "test" / "data"
    for name in ("standard_output_sum", "standard_output_sum_custom_shape"):
        arr = read_tiff(data / f"{name}.tif")
        np.save(HERE / f"{name}.npy", arr)
        print(name, arr.shape, arr.dtype, int((arr > 0).sum()))
    geoms = read_geoms(ref_root / "python" / "test" / "test_many.py")
    spec = {
        "source": "python/test/test_many.py:19-28 (GEOMS, value = 1..len(GEOMS))",
        "geoms": geoms,
        "values": list(range(1, len(geoms) + 1)),
    }
    (HERE / "golden_inputs.json").write_text(json.dumps(spec, indent=1) + "\n")
    print("geoms", len(geoms))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of a ttrotto/rusterize checkout>")
    main(Path(sys.argv[1]))
