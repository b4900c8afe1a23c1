"""Writes Ewald table files in the layout of the reference's
save_t3_ewald_lookup_table / save_s1r2_ewald_lookup_table
(StePS/src/inputoutput.cc:1792, :2102): a /Header group with the integer
attributes EWALD_GRID_SIZE (or EWALD_GRID_SIZE_RHO and EWALD_GRID_SIZE_Z) and
EWALD_PRECISION, and a /t3_ewald (or /s1r2_ewald) group holding the table as
a contiguous (Ng, Ng, Ng, 3) (or (Nrho, Nz, 2)) dataset of little-endian
IEEE doubles (floats for a single-precision build).

The files use the structures the HDF5 library writes with default
properties (superblock version 0, version 1 object headers, symbol-table
groups, contiguous storage), written out by hand after the published HDF5
file format specification, since no HDF5 installation is available here.
The table values are the reference's own tables from the golden set, so a
loader test compares the loaded table with them bit for bit.

    python tests/golden/make_h5_tables.py   # writes tests/golden/*.h5
"""
from __future__ import annotations

import os
import struct

import numpy as np

GOLDEN = os.path.dirname(os.path.abspath(__file__))
UNDEF = 0xFFFFFFFFFFFFFFFF


class Writer:
    """Appends structures to a byte buffer; every structure starts on an 8-byte boundary."""

    def __init__(self):
        self.b = bytearray(96)  # superblock + root symbol table entry, patched at the end

    def put(self, data: bytes) -> int:
        while len(self.b) % 8:
            self.b.append(0)
        at = len(self.b)
        self.b += data
        return at

    def patch(self, at: int, data: bytes):
        self.b[at:at + len(data)] = data


def message(mtype: int, data: bytes) -> bytes:
    data = data + b"\0" * (-len(data) % 8)
    return struct.pack("<HHB3x", mtype, len(data), 0) + data


def object_header(messages: list[bytes]) -> bytes:
    body = b"".join(messages)
    return struct.pack("<BBHII", 1, 0, len(messages), 1, len(body)) + b"\0" * 4 + body


def dataspace(dims) -> bytes:
    return struct.pack("<BBBB4x", 1, len(dims), 0, 0) + b"".join(struct.pack("<Q", d) for d in dims)


def float_type(size: int) -> bytes:
    # class 1 (floating point), version 1; little endian, IEEE mantissa normalisation
    if size == 8:
        return struct.pack("<BBBBI", 0x11, 0x20, 0x3F, 0x00, 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    return struct.pack("<BBBBI", 0x11, 0x20, 0x1F, 0x00, 4) + struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)


def int32_type() -> bytes:
    # class 0 (fixed point), version 1; little endian, signed
    return struct.pack("<BBBBI", 0x10, 0x08, 0x00, 0x00, 4) + struct.pack("<HH", 0, 32)


def attribute(name: str, value: int) -> bytes:
    nm = name.encode() + b"\0"
    dt, ds = int32_type(), struct.pack("<BBBB4x", 1, 0, 0, 0)  # scalar dataspace

    def pad(x):
        return x + b"\0" * (-len(x) % 8)

    return message(0x0C, struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds)) + pad(nm) + pad(dt) + pad(ds) +
                   struct.pack("<i", value))


def symbol_group(w: Writer, entries: list[tuple[str, int]], extra: list[bytes] = ()) -> int:
    """A group whose members are (name, object header address); returns its object header address."""
    names = sorted(entries)
    heap_data = bytearray(b"\0" * 8)  # offset 0: the empty name
    offs = []
    for n, _ in names:
        offs.append(len(heap_data))
        heap_data += n.encode() + b"\0"
        heap_data += b"\0" * (-len(heap_data) % 8)
    data_at = w.put(bytes(heap_data))
    heap_at = w.put(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), UNDEF, data_at))
    snod = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for (n, oh), off in zip(names, offs):
        snod += struct.pack("<QQII16x", off, oh, 0, 0)
    snod_at = w.put(snod)
    if names:
        tree = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, UNDEF, UNDEF) + struct.pack("<QQQ", 0, snod_at, offs[-1])
    else:
        tree = b"TREE" + struct.pack("<BBHQQ", 0, 0, 0, UNDEF, UNDEF) + struct.pack("<Q", 0)
    tree_at = w.put(tree)
    return w.put(object_header([message(0x11, struct.pack("<QQ", tree_at, heap_at))] + list(extra)))


def dataset(w: Writer, arr: np.ndarray) -> int:
    raw = np.ascontiguousarray(arr).astype(arr.dtype.newbyteorder("<")).tobytes()
    data_at = w.put(raw)
    layout = struct.pack("<BBQQ", 3, 1, data_at, len(raw))
    return w.put(object_header([message(0x01, dataspace(arr.shape)), message(0x03, float_type(arr.dtype.itemsize)),
                                message(0x08, layout)]))


def write_file(path: str, group: str, dset: str, arr: np.ndarray, attrs: dict[str, int]):
    w = Writer()
    header = symbol_group(w, [], [attribute(k, v) for k, v in attrs.items()])
    ds = dataset(w, arr)
    grp = symbol_group(w, [(dset, ds)])
    root = symbol_group(w, [("Header", header), (group, grp)])
    eof = len(w.b)
    sb = b"\x89HDF\r\n\x1a\n" + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, 4, 16, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sb += struct.pack("<QQII16x", 0, root, 0, 0)  # root group symbol table entry
    w.patch(0, sb)
    with open(path, "wb") as f:
        f.write(bytes(w.b))


def main():
    g = np.load(os.path.join(GOLDEN, "t3_o2.npz"))
    ng = int(g["ngrid"])
    t3 = np.asarray(g["table"], dtype=np.float64).reshape(ng, ng, ng, 3)
    write_file(os.path.join(GOLDEN, "t3_table_ng17.h5"), "t3_ewald", "T3_EWALD_FORCE_TABLE", t3,
               {"EWALD_GRID_SIZE": ng, "EWALD_PRECISION": 1})
    write_file(os.path.join(GOLDEN, "t3_table_ng17_f32.h5"), "t3_ewald", "T3_EWALD_FORCE_TABLE",
               t3.astype(np.float32), {"EWALD_GRID_SIZE": ng, "EWALD_PRECISION": 0})
    s = np.load(os.path.join(GOLDEN, "s1r2_table_o2.npz"))
    nrho, nz = (int(v) for v in s["shape"])
    s1 = np.asarray(s["table"], dtype=np.float64).reshape(nrho, nz, 2)
    write_file(os.path.join(GOLDEN, "s1r2_table.h5"), "s1r2_ewald", "S1R2_EWALD_FORCE_TABLE", s1,
               {"EWALD_GRID_SIZE_RHO": nrho, "EWALD_GRID_SIZE_Z": nz, "EWALD_PRECISION": 1})


if __name__ == "__main__":
    main()
