"""Matrix and geometry file formats of the reference, byte-compatible.

``.bin`` (``OpenMEEGMaths/include/TrivialBinIO.H:34-137``): a uint32 row
count, then a uint32 column count unless the matrix is symmetric or a vector,
then float64 payload -- column-major for full matrices, packed upper
(``i + j(j+1)/2``, ``OpenMEEGMaths/include/symmatrix.h:52-62``) for symmetric
ones, and ``(uint32 i, uint32 j, float64 v)`` triples for sparse ones.  The
type is inferred from the file size, as the reference does.

Text inputs: ``.tri`` meshes (``OpenMEEG/include/MeshIOs/tri.h``), ``.geom``
v1.1 (``OpenMEEG/include/GeometryIOs/GeomFile.h:165-300``), ``.cond``
(``OpenMEEG/src/geometry.cpp:231-252``), dipoles (n x 6) and sensors (3, 6 or 7
columns, ``OpenMEEG/src/sensors.cpp:36-120``).  Numbers are written with 17
significant digits and always carry a decimal point, so that the reference's
sensor loader never mistakes a value for a label.
"""
from __future__ import annotations

import os
import struct

import numpy as np

__all__ = ["read_bin", "write_bin", "packed_upper", "unpack_upper", "write_tri", "read_tri", "write_geom",
           "write_cond", "write_matrix_txt", "read_matrix_txt", "read_geom", "read_cond"]

_U32_MAX = 2**32 - 1


def packed_upper(M: np.ndarray) -> np.ndarray:
    """Dense symmetric -> packed upper column-major (SymMatrix storage)."""
    n = M.shape[0]
    iu = np.triu_indices(n)
    out = np.empty(n * (n + 1) // 2)
    out[iu[0] + iu[1] * (iu[1] + 1) // 2] = M[iu]
    return out


def unpack_upper(p: np.ndarray, n: int) -> np.ndarray:
    M = np.zeros((n, n))
    iu = np.triu_indices(n)
    M[iu] = p[iu[0] + iu[1] * (iu[1] + 1) // 2]
    return M + np.triu(M, 1).T


def write_bin(path: str, M, kind: str = "full") -> None:
    """kind: 'full' (2-D array), 'sym' (2-D symmetric array or packed 1-D with
    n given by shape), 'vector', or 'sparse' ((rows, cols, vals, nlin, ncol))."""
    with open(path, "wb") as f:
        if kind == "sym":
            M = np.asarray(M, np.float64)
            if M.ndim == 2:
                n = M.shape[0]
                data = packed_upper(M)
            else:
                n = int((np.sqrt(8 * M.size + 1) - 1) // 2)
                data = M
            if n > _U32_MAX:
                raise OverflowError("matrix too large for the .bin header")
            f.write(struct.pack("<I", n))
            f.write(np.ascontiguousarray(data, "<f8").tobytes())
        elif kind == "vector":
            v = np.asarray(M, np.float64).ravel()
            f.write(struct.pack("<I", v.size))
            f.write(v.astype("<f8").tobytes())
        elif kind == "sparse":
            rows, cols, vals, nlin, ncol = M
            f.write(struct.pack("<II", nlin, ncol))
            order = np.lexsort((np.asarray(cols), np.asarray(rows)))
            for k in order:
                f.write(struct.pack("<IId", int(rows[k]), int(cols[k]), float(vals[k])))
        else:
            M = np.asarray(M, np.float64)
            f.write(struct.pack("<II", M.shape[0], M.shape[1]))
            f.write(np.asfortranarray(M).astype("<f8").tobytes(order="F"))


def read_bin(path: str):
    """Returns (kind, array).  'sym' -> dense symmetric; 'sparse' -> dense."""
    b = open(path, "rb").read()
    size = len(b) - 4
    nlin = struct.unpack("<I", b[:4])[0]
    if size == nlin * 8:
        return "vector", np.frombuffer(b[4:], "<f8").copy()
    n = nlin
    if size == n * (n + 1) * 8 // 2:
        return "sym", unpack_upper(np.frombuffer(b[4:], "<f8"), n)
    ncol = struct.unpack("<I", b[4:8])[0]
    if size - 4 == nlin * ncol * 8:
        return "full", np.frombuffer(b[8:], "<f8").reshape((ncol, nlin)).T.copy()
    M = np.zeros((nlin, ncol))
    rec = np.frombuffer(b[8:], dtype=np.dtype([("i", "<u4"), ("j", "<u4"), ("v", "<f8")]))
    M[rec["i"], rec["j"]] = rec["v"]
    return "sparse", M


def _fmt(x: float) -> str:
    s = f"{x:.17e}"
    return s


def write_tri(path: str, V: np.ndarray, T: np.ndarray) -> None:
    """``.tri``: '- nv', lines 'x y z nx ny nz', '- nt nt nt', triangle lines."""
    nrm = V / np.linalg.norm(V, axis=1, keepdims=True)
    with open(path, "w") as f:
        f.write(f"- {V.shape[0]}\n")
        for v, n in zip(V, nrm):
            f.write(" ".join(_fmt(x) for x in (*v, *n)) + "\n")
        nt = T.shape[0]
        f.write(f"- {nt} {nt} {nt}\n")
        for t in T:
            f.write(f"{int(t[0])} {int(t[1])} {int(t[2])}\n")


def read_tri(path: str):
    with open(path) as f:
        tok = f.read().split()
    assert tok[0] == "-"
    nv = int(tok[1])
    vals = np.array(tok[2:2 + 6 * nv], dtype=np.float64).reshape(nv, 6)
    k = 2 + 6 * nv
    assert tok[k] == "-"
    nt = int(tok[k + 1])
    T = np.array(tok[k + 4:k + 4 + 3 * nt], dtype=np.int64).reshape(nt, 3)
    return vals[:, :3].copy(), T


def write_geom(path: str, mesh_files, domains) -> None:
    """``.geom`` v1.1 with meshes given as interfaces; domains as
    (name, [signed 1-based interface ids], sigma)."""
    with open(path, "w") as f:
        f.write("# Domain Description 1.1\n\n")
        f.write(f"Interfaces {len(mesh_files)}\n\n")
        for mf in mesh_files:
            f.write(f'Interface: "{mf}"\n')
        f.write(f"\nDomains {len(domains)}\n\n")
        for (name, bounds, _) in domains:
            f.write(f"Domain {name}: " + " ".join(str(b) for b in bounds) + "\n")


def write_cond(path: str, domains) -> None:
    with open(path, "w") as f:
        f.write("# Properties Description 1.0 (Conductivities)\n\n")
        for (name, _, sigma) in domains:
            f.write(f"{name} {_fmt(sigma)}\n")


def read_geom(path: str):
    """Parse a ``.geom`` v1.1 file whose interfaces are single meshes.
    Returns (mesh_paths, domains without conductivities)."""
    base = os.path.dirname(os.path.abspath(path))
    lines = [ln.split("#", 1)[0].strip() if not ln.lstrip().startswith("#") else ""
             for ln in open(path).read().splitlines()]
    head = open(path).readline()
    if "1.1" not in head:
        raise ValueError("only .geom version 1.1 is supported")
    lines = [ln for ln in lines if ln]
    meshes, domains = [], []
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("Interfaces"):
            n = int(ln.split()[1])
            for k in range(n):
                i += 1
                ent = lines[i]
                fn = ent.split('"')[1] if '"' in ent else ent.split()[-1]
                meshes.append(fn if os.path.isabs(fn) else os.path.join(base, fn))
        elif ln.startswith("Domains"):
            n = int(ln.split()[1])
            for k in range(n):
                i += 1
                ent = lines[i][len("Domain"):].strip()
                name, rest = ent.split(":", 1) if ":" in ent else (ent.split()[0], " ".join(ent.split()[1:]))
                bounds = [int(t) for t in rest.split() if t != "shared"]
                domains.append((name.strip(), bounds))
        i += 1
    return meshes, domains


def read_cond(path: str) -> dict:
    out = {}
    for ln in open(path):
        ln = ln.split("#", 1)[0].strip()
        if ln:
            name, val = ln.split()[:2]
            out[name] = float(val)
    return out


def write_matrix_txt(path: str, M: np.ndarray) -> None:
    with open(path, "w") as f:
        for row in np.atleast_2d(M):
            f.write(" ".join(_fmt(x) for x in row) + "\n")


def read_matrix_txt(path: str) -> np.ndarray:
    rows = []
    for ln in open(path):
        ln = ln.split("#", 1)[0].strip()
        if ln:
            tok = ln.split()
            if tok[0].count(".") != 1:  # labelled line
                tok = tok[1:]
            rows.append([float(t) for t in tok])
    return np.array(rows, dtype=np.float64)
