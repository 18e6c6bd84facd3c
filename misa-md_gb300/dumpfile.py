"""Reader of the binary atom dumps that mg_dump_* writes (the reference's copy-mode layout of one rank,
frontend/io/atom_dump.cpp:38-82 as tools/dump2text/out_convert.cpp reads it).

File: 128-byte file header (zeros), 128-byte rank header whose first 8 bytes are the record count, then
72-byte records {id u64, step u64, type i32, inter_type i16, pad, x f64[3], v f64[3]}. A single-file
dump holds its frames one after another; `frames()` splits them by time step.
"""
from __future__ import annotations

import numpy as np

RECORD_DTYPE = np.dtype(
    [("id", "<u8"), ("step", "<u8"), ("type", "<i4"), ("inter_type", "<i2"), ("pad_", "<i2"),
     ("x", "<f8", (3,)), ("v", "<f8", (3,))],
    align=True,
)
HEADER_BYTES = 128 + 128
TYPE_NAMES = {0: "Fe", 1: "Cu", 2: "Ni"}   # getNameByEleName, out_convert.cpp:171-182


def read(path) -> np.ndarray:
    """All records of a dump file, in file order."""
    with open(path, "rb") as f:
        head = f.read(HEADER_BYTES)
        if len(head) != HEADER_BYTES:
            raise ValueError(f"{path}: shorter than the dump header")
        count = int(np.frombuffer(head[128:136], dtype="<u8")[0])
        recs = np.fromfile(f, dtype=RECORD_DTYPE, count=count)
    if recs.size != count:
        raise ValueError(f"{path}: {recs.size} records for a header count of {count}")
    return recs


def frames(path) -> dict:
    """{time step: records of that frame} of a dump file (frames keep their file order)."""
    recs = read(path)
    if recs.size == 0:
        return {}
    cut = np.flatnonzero(np.diff(recs["step"].astype(np.int64))) + 1
    return {int(part["step"][0]): part for part in np.split(recs, cut)}
