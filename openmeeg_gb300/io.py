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
           "write_cond", "write_matrix_txt", "read_matrix_txt", "read_sensors_txt", "read_geom", "read_geom_full",
           "read_cond",
           "read_off", "read_mesh", "load_head"]

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


def read_off(path: str):
    """OFF mesh (MeshIOs/off.h): 'OFF', 'nv nt 0', vertices, faces '3 i j k'."""
    with open(path) as f:
        tok = [t for ln in f for t in ln.split("#", 1)[0].split()]
    if tok[0] != "OFF":
        raise ValueError(f"{path}: not an OFF file")
    nv, nt = int(tok[1]), int(tok[2])
    V = np.array(tok[4:4 + 3 * nv], dtype=np.float64).reshape(nv, 3)
    F = np.array(tok[4 + 3 * nv:4 + 3 * nv + 4 * nt], dtype=np.int64).reshape(nt, 4)
    if np.any(F[:, 0] != 3):
        raise ValueError(f"{path}: OFF faces must be triangles")
    return V, F[:, 1:].copy()


def read_mesh(path: str):
    """A .tri or .off mesh: (vertices n x 3, triangles m x 3, 0-based)."""
    if path.endswith(".tri"):
        return read_tri(path)
    if path.endswith(".off"):
        return read_off(path)
    raise ValueError(f"{path}: only .tri and .off meshes are supported")


def _entry(line: str, keyword: str, index: int):
    """('Keyword name: rest' | 'Keyword: rest' | 'rest') -> (name, rest); unnamed entries are
    named by their position, 1-based (GeomFile.h:87-91, 114-119)."""
    s = line.strip()
    if s.startswith(keyword):
        after = s[len(keyword):]
        if ":" in after:
            name, rest = after.split(":", 1)
            return (name.strip() or str(index + 1)), rest
    return str(index + 1), s


def _fname(rest: str, base: str) -> str:
    fn = rest.split('"')[1] if '"' in rest else rest.split()[0]
    return fn if os.path.isabs(fn) else os.path.join(base, fn)


def read_geom_full(path: str):
    """Parse a ``.geom`` v1.1 file (GeomFile.h:160-300): an optional "Meshes"
    section, "Interfaces" given as mesh files or as lists of +/-mesh names, and
    "Domains" as lists of +/-interface names ('-' = inside).  Returns
    (meshes [(name, path)], interfaces [(name, [(mesh index, +1/-1)])],
    domains [(name, [(interface index, inside)])])."""
    base = os.path.dirname(os.path.abspath(path))
    head = open(path).readline()
    if "1.1" not in head:
        raise ValueError("only .geom version 1.1 is supported")
    lines = [ln.split("#", 1)[0].strip() for ln in open(path).read().splitlines()]
    lines = [ln for ln in lines if ln]
    meshes, ifaces, domains = [], [], []
    mesh_section = False
    i = 0
    while i < len(lines):
        key = lines[i].split()[0]
        if key == "MeshFile":
            raise ValueError("geometries given as one mesh file (MeshFile) are not supported")
        if key == "Meshes":
            mesh_section = True
            for k in range(int(lines[i].split()[1])):
                i += 1
                name, rest = _entry(lines[i], "Mesh", k)
                meshes.append((name, _fname(rest, base)))
        elif key == "Interfaces":
            for k in range(int(lines[i].split()[1])):
                i += 1
                name, rest = _entry(lines[i], "Interface", k)
                if not mesh_section:
                    meshes.append((name, _fname(rest, base)))
                    ifaces.append((name, [(len(meshes) - 1, 1)]))
                else:
                    om = []
                    for t in rest.split():
                        sign = -1 if t[0] == "-" else 1
                        t = t[1:] if t[0] in "+-" else t
                        om.append(([m[0] for m in meshes].index(t), sign))
                    ifaces.append((name, om))
        elif key == "Domains":
            for k in range(int(lines[i].split()[1])):
                i += 1
                name, rest = _entry(lines[i], "Domain", k)
                b = []
                for t in rest.split():
                    if t == "shared":
                        break
                    inside = t[0] == "-"
                    t = t[1:] if t[0] in "+-" else t
                    b.append(([f[0] for f in ifaces].index(t), inside))
                domains.append((name, b))
        i += 1
    return meshes, ifaces, domains


def read_geom(path: str):
    """A ``.geom`` v1.1 file whose interfaces are single meshes: (mesh paths,
    domains as (name, [signed 1-based mesh ids])), '-' = inside."""
    meshes, ifaces, domains = read_geom_full(path)
    for name, om in ifaces:
        if len(om) != 1:
            raise ValueError(f"interface {name} is made of several meshes")
    doms = [(name, [-(ifaces[k][1][0][0] + 1) if inside else ifaces[k][1][0][0] + 1 for k, inside in b])
            for name, b in domains]
    return [p for _, p in meshes], doms


def load_head(geom_path: str, cond_path: str):
    """Meshes, names and domains (with conductivities) of a .geom/.cond pair, as
    the head description that ``Geometry.from_head`` and the oracle take."""
    from .synthetic import NestedHead
    meshes, ifaces, _ = read_geom_full(geom_path)
    paths, doms = read_geom(geom_path)
    cond = read_cond(cond_path)
    V, T = zip(*[read_mesh(p) for p in paths])
    return NestedHead(list(V), list(T), [n for n, _ in meshes], [(n, b, cond[n]) for n, b in doms])


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
    """A plain numeric text matrix (dipole files and the like; the reference's
    ASCII Matrix reader): one row per non-empty line, '#' comments."""
    rows = []
    for ln in open(path):
        ln = ln.split("#", 1)[0].strip()
        if ln:
            rows.append([float(t) for t in ln.split()])
    return np.array(rows, dtype=np.float64)


def read_sensors_txt(path: str):
    """A sensors file (Sensors::load, sensors.cpp:36-120): the lines are
    labelled unless the first token of some line is a number with exactly one
    '.'; labels, when present, are the first token of every line.  Returns
    (labels or None, values n x columns)."""
    lines = [ln.split("#", 1)[0].split() for ln in open(path)]
    lines = [t for t in lines if t]
    labeled = not any(t[0].count(".") == 1 for t in lines)
    if labeled:
        return [t[0] for t in lines], np.array([[float(x) for x in t[1:]] for t in lines], dtype=np.float64)
    return None, np.array([[float(x) for x in t] for t in lines], dtype=np.float64)
