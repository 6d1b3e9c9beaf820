"""Test-side restatement of the reference's param(81)=3 VTK writer
(src/io_vtkbin.c writeheader/writenodes/write3dcells/writefield, fields of
cem_out_fields3 in src/io.F:562-640, cell numbering of
vtk_dump_header_nonswap in src/io_dumpvtk.F:718-810): big-endian binary, FP32
points and vectors.  Used to check the library's writer byte for byte."""
from __future__ import annotations

import numpy as np


def cells(n: int, nelt: int) -> np.ndarray:
    out = []
    for e in range(nelt):
        for j in range(1, n):
            cnt = (j - 1) * n * n + e * n ** 3
            for _ in range((n - 1) * (n - 1)):
                v = [cnt, cnt + 1, cnt + n + 1, cnt + n]
                out.append(v + [x + n * n for x in v])
                cnt += 1
                if (cnt + 1) % n == 0:
                    cnt += 1
    return np.array(out, dtype=np.int64)


def vtk_bytes(x, y, z, n, nelt, H, E, solH=None, solE=None) -> bytes:
    npts = x.size
    b = bytearray()
    b += b"# vtk DataFile Version 2.0 \n"
    b += b"Electromagnetic Field  \n"
    b += b"BINARY \n"
    b += b"DATASET UNSTRUCTURED_GRID \n"
    b += f"POINTS  {npts} ".encode() + b" float  \n"
    b += np.stack([x, y, z], axis=1).astype(">f4").tobytes()
    b += b" \n"
    cl = cells(n, nelt)
    b += f"CELLS {len(cl)}  {9 * len(cl)} \n".encode()
    b += np.concatenate([np.full((len(cl), 1), 8), cl], axis=1).astype(">i4").tobytes()
    b += b"\n"
    b += f"CELL_TYPES {len(cl)} \n".encode()
    b += np.full(len(cl), 12).astype(">i4").tobytes()
    b += b"\n"
    b += f"POINT_DATA {npts} \n".encode()
    fields = [("E ", E), ("H ", H)]
    if solH is not None:
        fields += [("solE", solE), ("solH", solH)]
    for name, f in fields:
        b += f"VECTORS {name} ".encode() + b" float \n"
        b += np.asarray(f).T.astype(">f4").tobytes()
        b += b" \n"
    return bytes(b)
