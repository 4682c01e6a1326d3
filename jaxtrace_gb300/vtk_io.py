"""VTK XML unstructured-grid time series without the VTK library.

Reads what VTKUnstructuredTimeSeriesReader (io/vtk_reader.py:426-940) reads
through VTK -- serial ``.vtu`` and parallel ``.pvtu`` files, one per time step
-- with a direct XML / appended-binary parser, and returns the same
JAXTrace-format dictionary: velocity_data (T, N, 3) float32, positions (N, 3)
float32, times = step indices (vtk_reader.py:697-765).  ``tetrahedra()`` gives
the VTK_TETRA cells as (M, 4) int32 for the FEM fields.

DataArray encodings: ascii, binary (base64) and appended raw data, UInt32
or UInt64 headers, optionally vtkZLibDataCompressor blocks (base64-encoded
appended data is refused).
``write_vtu`` writes the same format (appended raw, base64 or ascii) for
exporting trajectories and for tests.
"""
from __future__ import annotations

import base64
import glob
import os
import re
import warnings
import xml.etree.ElementTree as ET
import zlib
from typing import Any, Dict, List, Optional, Tuple

import numpy as np

F32 = np.float32
VTK_VERTEX = 1
VTK_TETRA = 10

_TYPES = {"Int8": np.int8, "UInt8": np.uint8, "Int16": np.int16, "UInt16": np.uint16, "Int32": np.int32,
          "UInt32": np.uint32, "Int64": np.int64, "UInt64": np.uint64, "Float32": np.float32,
          "Float64": np.float64}
_NAMES = {np.dtype(v): k for k, v in _TYPES.items()}

# velocity field names tried in order when none is given (vtk_reader.py:565-575)
VELOCITY_NAMES = ["velocity", "Velocity", "VELOCITY", "U", "u", "vel", "Vel", "VEL", "Displacement",
                  "displacement", "DISPLACEMENT", "VelocityField", "velocity_field", "FlowVelocity",
                  "flow_velocity", "v", "V", "fluid_velocity", "Result", "RESULT", "NodeVel", "NODEVEL"]


def _natural_key(path: str) -> tuple:
    nums = tuple(int(x) for x in re.findall(r"\d+", os.path.basename(path)))
    return nums if nums else (os.path.basename(path),)


class _Blob:
    """The decoding context of one XML file: byte order, header type,
    compressor and the appended-data block."""

    def __init__(self, root: ET.Element, raw: bytes, app_at: int):
        self.little = root.get("byte_order", "LittleEndian") == "LittleEndian"
        self.header = np.dtype(np.uint64 if root.get("header_type", "UInt32") == "UInt64" else np.uint32)
        self.compressed = root.get("compressor", "") == "vtkZLibDataCompressor"
        self.appended = b""
        self.appended_b64 = False
        if app_at >= 0:
            tag_end = raw.find(b">", app_at)
            self.appended_b64 = b'encoding="base64"' in raw[app_at:tag_end]
            # the bytes start after the '_' marker that follows the tag
            j = raw.find(b"_", tag_end) + 1
            end = raw.rfind(b"</AppendedData>")
            self.appended = raw[j:end]

    def _hdr(self) -> np.dtype:
        return self.header.newbyteorder("<" if self.little else ">")

    def _payload(self, data: bytes) -> bytes:
        """One binary DataArray (header + data, or compressed blocks)."""
        h = self._hdr()
        hs = h.itemsize
        if not self.compressed:
            n = int(np.frombuffer(data[:hs], dtype=h)[0])
            return data[hs:hs + n]
        nb = int(np.frombuffer(data[:hs], dtype=h)[0])
        head = np.frombuffer(data[:hs * (3 + nb)], dtype=h).astype(np.int64)
        sizes = head[3:3 + nb]
        pos = hs * (3 + nb)
        out = []
        for s in sizes:
            out.append(zlib.decompress(data[pos:pos + int(s)]))
            pos += int(s)
        return b"".join(out)

    def array(self, el: ET.Element) -> np.ndarray:
        dt = np.dtype(_TYPES[el.get("type")]).newbyteorder("<" if self.little else ">")
        ncomp = int(el.get("NumberOfComponents", "1"))
        fmt = el.get("format", "ascii")
        if fmt == "ascii":
            a = np.array((el.text or "").split(), dtype=dt.newbyteorder("="))
        elif fmt == "binary":
            text = "".join((el.text or "").split()).encode()
            if self.compressed:
                # base64 of the header, then base64 of the compressed blocks
                hs = self._hdr().itemsize
                first = base64.b64decode(text[:((hs + 2) // 3) * 4])
                nb = int(np.frombuffer(first[:hs], dtype=self._hdr())[0])
                hlen = ((hs * (3 + nb) + 2) // 3) * 4
                head = base64.b64decode(text[:hlen])[: hs * (3 + nb)]
                body = base64.b64decode(text[hlen:])
                a = np.frombuffer(self._payload(head + body), dtype=dt)
            else:
                a = np.frombuffer(self._payload(base64.b64decode(text)), dtype=dt)
        elif fmt == "appended":
            off = int(el.get("offset", "0"))
            if self.appended_b64:
                raise NotImplementedError("base64-encoded appended data is not supported; use raw or binary")
            a = np.frombuffer(self._payload(self.appended[off:]), dtype=dt)
        else:
            raise ValueError(f"unknown DataArray format {fmt!r}")
        a = a.astype(dt.newbyteorder("="), copy=False)
        return a.reshape(-1, ncomp) if ncomp > 1 else a


def _read_piece(path: str, geometry: bool = True, names: Optional[List[str]] = None) -> Dict[str, Any]:
    """One .vtu (or .vtp) file; without ``geometry`` the points and cells
    are left undecoded, and with ``names`` only those point arrays are
    decoded.  PolyData cells come as {"verts": {...}, "lines": {...}}."""
    raw = open(path, "rb").read()
    # raw appended data is not XML: parse the part before it, closed
    app_at = raw.find(b"<AppendedData")
    root = ET.fromstring(raw if app_at < 0 else raw[:app_at] + b"</VTKFile>")
    kind = root.get("type")
    if kind not in ("UnstructuredGrid", "PolyData"):
        raise ValueError(f"{path}: not an UnstructuredGrid or PolyData file ({kind})")
    blob = _Blob(root, raw, app_at)
    piece = root.find(f"{kind}/Piece")
    n_points = int(piece.get("NumberOfPoints", "0"))
    pts, cells = None, {}
    if geometry:
        pts = np.asarray(blob.array(piece.find("Points/DataArray")), dtype=F32).reshape(-1, 3)
        if kind == "UnstructuredGrid":
            for el in piece.findall("Cells/DataArray"):
                cells[el.get("Name")] = blob.array(el)
        else:
            for sec in ("Verts", "Lines", "Strips", "Polys"):
                d = {el.get("Name"): blob.array(el) for el in piece.findall(f"{sec}/DataArray")}
                if d:
                    cells[sec.lower()] = d
    pdata = {}
    pd = piece.find("PointData")
    if pd is not None:
        for el in pd.findall("DataArray"):
            if names is None or el.get("Name") in names:
                pdata[el.get("Name")] = blob.array(el)
            else:
                pdata[el.get("Name")] = None          # present, not decoded
    cdata = {el.get("Name"): blob.array(el) for el in piece.findall("CellData/DataArray")}
    return {"points": pts, "n_points": n_points, "cells": cells, "point_data": pdata, "cell_data": cdata}


_LEGACY_TYPES = {"float": ">f4", "double": ">f8", "int": ">i4", "unsigned_int": ">u4", "long": ">i8",
                 "unsigned_long": ">u8", "short": ">i2", "unsigned_short": ">u2", "char": ">i1",
                 "unsigned_char": ">u1", "vtktypeint64": ">i8", "vtktypeint32": ">i4", "vtkidtype": ">i8"}


class _Legacy:
    """Cursor over a legacy VTK file: header lines and ASCII or big-endian
    binary value blocks."""

    def __init__(self, raw: bytes):
        self.raw, self.pos, self.binary = raw, 0, False

    def line(self, skip_blank: bool = True) -> Optional[str]:
        while self.pos < len(self.raw):
            end = self.raw.find(b"\n", self.pos)
            end = len(self.raw) if end < 0 else end
            text = self.raw[self.pos:end].decode("latin-1").strip()
            self.pos = end + 1
            if text or not skip_blank:
                return text
        return None

    def values(self, count: int, vtype: str) -> np.ndarray:
        dt = np.dtype(_LEGACY_TYPES.get(vtype.lower(), ""))
        if self.binary:
            nb = count * dt.itemsize
            a = np.frombuffer(self.raw, dtype=dt, count=count, offset=self.pos)
            self.pos += nb
            if self.raw[self.pos:self.pos + 1] == b"\n":
                self.pos += 1
            return a.astype(dt.newbyteorder("="))
        toks: List[bytes] = []
        while len(toks) < count:
            end = self.raw.find(b"\n", self.pos)
            end = len(self.raw) if end < 0 else end
            toks += self.raw[self.pos:end].split()
            self.pos = end + 1
            if end >= len(self.raw) and len(toks) < count:
                raise ValueError("legacy VTK file ends inside a data block")
        return np.array(toks[:count], dtype=dt.newbyteorder("="))


def _read_legacy(path: str, geometry: bool = True, names: Optional[List[str]] = None) -> Dict[str, Any]:
    """A legacy .vtk UNSTRUCTURED_GRID (what vtkUnstructuredGridReader reads,
    io/vtk_reader.py:633-634): ASCII or BINARY, classic CELLS or the 5.1
    OFFSETS/CONNECTIVITY layout, point arrays from SCALARS, VECTORS, NORMALS
    and FIELD blocks; METADATA blocks are skipped."""
    cur = _Legacy(open(path, "rb").read())
    if not (cur.line() or "").lower().startswith("# vtk datafile"):
        raise ValueError(f"{path}: not a legacy VTK file")
    cur.line(skip_blank=False)                       # title
    cur.binary = (cur.line() or "").upper() == "BINARY"
    ds = (cur.line() or "").split()
    if len(ds) < 2 or ds[0].upper() != "DATASET" or ds[1].upper() != "UNSTRUCTURED_GRID":
        raise ValueError(f"{path}: only DATASET UNSTRUCTURED_GRID is read ({' '.join(ds)})")
    pts, cells, pdata, cdata = None, {}, {}, {}
    n_points, target = 0, None
    while True:
        ln = cur.line()
        if ln is None:
            break
        tok = ln.split()
        key = tok[0].upper()
        if key == "METADATA":
            while cur.line(skip_blank=False):
                pass
        elif key == "POINTS":
            n_points = int(tok[1])
            pts = cur.values(3 * n_points, tok[2]).astype(F32).reshape(-1, 3)
        elif key == "CELLS":
            n0, n1 = int(tok[1]), int(tok[2])
            nxt = cur.pos
            sub = (cur.line() or "").split()
            if sub and sub[0].upper() == "OFFSETS":        # 5.1 layout: n0 offsets, n1 ids
                offs = cur.values(n0, sub[1]).astype(np.int64)
                sub = (cur.line() or "").split()
                conn = cur.values(n1, sub[1]).astype(np.int64)
                cells.update(connectivity=conn, offsets=offs[1:])
            else:                                          # classic: n0 records, n1 ints
                cur.pos = nxt
                rec = cur.values(n1, "int").astype(np.int64)
                ks, at = [], 0
                while at < len(rec):
                    ks.append(at)
                    at += int(rec[at]) + 1
                ks = np.array(ks, dtype=np.int64)
                cnt = rec[ks]
                keep = np.ones(len(rec), bool)
                keep[ks] = False
                cells.update(connectivity=rec[keep], offsets=np.cumsum(cnt))
        elif key == "CELL_TYPES":
            cells["types"] = cur.values(int(tok[1]), "int").astype(np.uint8)
        elif key in ("POINT_DATA", "CELL_DATA"):
            target = (pdata, int(tok[1])) if key == "POINT_DATA" else (cdata, int(tok[1]))
        elif key in ("SCALARS", "VECTORS", "NORMALS") and target is not None:
            d, n = target
            nc = (int(tok[3]) if len(tok) > 3 else 1) if key == "SCALARS" else 3
            if key == "SCALARS":
                lt = cur.pos
                if not (cur.line() or "").upper().startswith("LOOKUP_TABLE"):
                    cur.pos = lt
            a = cur.values(n * nc, tok[2])
            d[tok[1]] = a.reshape(n, nc) if nc > 1 else a
        elif key == "FIELD" and target is not None:
            d, _ = target
            for _ in range(int(tok[2])):
                ft = (cur.line() or "").split()
                while ft and ft[0].upper() == "METADATA":
                    while cur.line(skip_blank=False):
                        pass
                    ft = (cur.line() or "").split()
                nm, nc, nt = ft[0], int(ft[1]), int(ft[2])
                a = cur.values(nc * nt, ft[3])
                d[nm] = a.reshape(nt, nc) if nc > 1 else a
        elif key == "LOOKUP_TABLE":
            cur.values(4 * int(tok[2]), "float")
        else:
            raise ValueError(f"{path}: unsupported legacy VTK section {tok[0]!r}")
    if names is not None:
        pdata = {k: (v if k in names else None) for k, v in pdata.items()}
    return {"points": pts if geometry else None, "n_points": n_points, "cells": cells if geometry else {},
            "point_data": pdata, "cell_data": cdata}


def write_vtk_legacy(path: str, points: np.ndarray, tets: Optional[np.ndarray] = None,
                     point_data: Optional[Dict[str, np.ndarray]] = None, binary: bool = True,
                     layout: str = "classic") -> None:
    """A legacy .vtk UNSTRUCTURED_GRID of tetrahedra with point data (1- or
    3-component arrays as SCALARS / VECTORS, others in a FIELD block);
    ``layout`` "classic" (CELLS n size) or "5.1" (OFFSETS/CONNECTIVITY)."""
    pts = np.ascontiguousarray(points, dtype=F32).reshape(-1, 3)
    t4 = np.zeros((0, 4), np.int64) if tets is None else np.asarray(tets, dtype=np.int64).reshape(-1, 4)
    out = [f"# vtk DataFile Version {'5.1' if layout == '5.1' else '3.0'}\nwritten by jaxtrace_gb300\n"
           f"{'BINARY' if binary else 'ASCII'}\nDATASET UNSTRUCTURED_GRID\n".encode()]

    def block(a: np.ndarray, be: str) -> bytes:
        if binary:
            return np.ascontiguousarray(a).astype(be).tobytes() + b"\n"
        flat = a.reshape(-1).tolist()
        return (" ".join(repr(x) if a.dtype.kind == "f" else str(x) for x in flat) + "\n").encode()

    out.append(f"POINTS {len(pts)} float\n".encode() + block(pts, ">f4"))
    if layout == "5.1":
        offs = 4 * np.arange(len(t4) + 1, dtype=np.int64)
        out.append(f"CELLS {len(offs)} {t4.size}\nOFFSETS vtktypeint64\n".encode() + block(offs, ">i8"))
        out.append(b"CONNECTIVITY vtktypeint64\n" + block(t4.reshape(-1), ">i8"))
    else:
        rec = np.concatenate([np.full((len(t4), 1), 4, np.int64), t4], axis=1).astype(np.int32)
        out.append(f"CELLS {len(t4)} {rec.size}\n".encode() + block(rec, ">i4"))
    out.append(f"CELL_TYPES {len(t4)}\n".encode() + block(np.full(len(t4), VTK_TETRA, np.int32), ">i4"))
    fields = []
    if point_data:
        out.append(f"POINT_DATA {len(pts)}\n".encode())
        for k, v in point_data.items():
            v = np.asarray(v)
            nc = v.shape[1] if v.ndim > 1 else 1
            tname, be = ("float", ">f4") if v.dtype.kind == "f" else ("int", ">i4")
            if nc == 3 and v.dtype.kind == "f":
                out.append(f"VECTORS {k} {tname}\n".encode() + block(v.astype(be[1:]), be))
            elif nc == 1:
                out.append(f"SCALARS {k} {tname} 1\nLOOKUP_TABLE default\n".encode() + block(v.astype(be[1:]), be))
            else:
                fields.append((k, v, nc, tname, be))
        if fields:
            out.append(f"FIELD FieldData {len(fields)}\n".encode())
            for k, v, nc, tname, be in fields:
                out.append(f"{k} {nc} {len(v)} {tname}\n".encode() + block(v.astype(be[1:]), be))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))


def read_vtk_xml(path: str, geometry: bool = True, names: Optional[List[str]] = None) -> Dict[str, Any]:
    """points (N,3) float32, cells {connectivity, offsets, types} and
    point_data {name: (N,) or (N,C)} of a .vtu (or .vtp, or legacy .vtk) file, or of a .pvtu file's
    pieces appended in order (point ids of later pieces shifted).  Without
    ``geometry`` points and cells are skipped; with ``names`` only those
    point arrays are decoded (the others map to None)."""
    if path.lower().endswith(".vtk"):
        return _read_legacy(path, geometry, names)
    if not path.lower().endswith(".pvtu"):
        return _read_piece(path, geometry, names)
    root = ET.parse(path).getroot()
    base = os.path.dirname(path)
    pieces = [_read_piece(os.path.join(base, p.get("Source")), geometry, names)
              for p in root.findall("PUnstructuredGrid/Piece")]
    if not pieces:
        raise ValueError(f"{path}: no pieces")
    pts, conn, offs, types, pdata, shift, oshift = [], [], [], [], {}, 0, 0
    for p in pieces:
        if geometry:
            pts.append(p["points"])
            c = p["cells"]
            if "connectivity" in c:
                conn.append(np.asarray(c["connectivity"], dtype=np.int64) + shift)
                offs.append(np.asarray(c["offsets"], dtype=np.int64) + oshift)
                types.append(np.asarray(c["types"], dtype=np.uint8))
                oshift += len(c["connectivity"])
        shift += p["n_points"]
        for k, v in p["point_data"].items():
            pdata.setdefault(k, []).append(v)
    cells = {}
    if conn:
        cells = {"connectivity": np.concatenate(conn), "offsets": np.concatenate(offs),
                 "types": np.concatenate(types)}
    return {"points": np.concatenate(pts) if geometry else None, "n_points": shift, "cells": cells,
            "point_data": {k: (None if any(x is None for x in v) else np.concatenate(v)) for k, v in pdata.items()}}


def _velocity3(v: np.ndarray) -> np.ndarray:
    """(N, 3) float32 from an (N, components) array (_ensure_3d_velocity,
    vtk_reader.py:77-103): zero-padded or cut to three components.  A
    one-component array reads as 1-D, as vtk_to_numpy returns it, and is
    refused like the reference refuses it."""
    v = np.asarray(v, dtype=F32)
    if v.ndim != 2:
        raise ValueError(f"Velocity must be 2D array (N, D), got shape {v.shape}")
    if v.shape[1] < 3:
        v = np.concatenate([v, np.zeros((len(v), 3 - v.shape[1]), dtype=F32)], axis=1)
    return np.ascontiguousarray(v[:, :3])


class VTKUnstructuredTimeSeriesReader:
    """One .vtu/.pvtu per time step (vtk_reader.py:426-940): files matched by
    ``file_pattern``, .pvtu preferred over .vtu of the same name, naturally
    sorted; the last ``max_time_steps`` kept."""

    def __init__(self, file_pattern: str, max_time_steps: Optional[int] = None,
                 velocity_field_name: Optional[str] = None, cache_size_limit: Optional[int] = None):
        self.file_pattern = file_pattern
        self.max_time_steps = max_time_steps
        self.velocity_field_name = velocity_field_name
        self.cache_size_limit = 15 if cache_size_limit is None else int(cache_size_limit)
        self.time_files = self._find_time_files()
        if not self.time_files:
            raise ValueError(f"No VTK files found matching pattern: {file_pattern}")
        self.grid_points: Optional[np.ndarray] = None
        self._cells: Dict[str, np.ndarray] = {}
        self.velocity_cache: Dict[int, np.ndarray] = {}

    def _find_time_files(self) -> List[str]:
        if isinstance(self.file_pattern, (list, tuple)):       # an explicit file list (open_dataset)
            files = [os.path.expanduser(f) for f in self.file_pattern]
        else:
            files = glob.glob(os.path.expanduser(self.file_pattern))
        pvtu = [f for f in files if f.lower().endswith(".pvtu")]
        vtu = [f for f in files if f.lower().endswith(".vtu")]
        # legacy .vtk files (read by read_vtk_xml) when there is no XML file
        vtk = [f for f in files if f.lower().endswith(".vtk")]
        chosen = pvtu if pvtu else (vtu if vtu else vtk)
        chosen.sort(key=_natural_key)
        if self.max_time_steps is not None and len(chosen) > self.max_time_steps:
            chosen = chosen[-self.max_time_steps:]
        return chosen

    def __len__(self) -> int:
        return len(self.time_files)

    def _field_name(self, pdata: Dict[str, np.ndarray]) -> str:
        if self.velocity_field_name is not None:
            return self.velocity_field_name
        for name in VELOCITY_NAMES:
            if name in pdata:
                self.velocity_field_name = name
                return name
        avail = [f"{k} ({1 if np.ndim(a) < 2 else np.shape(a)[1]}D)" for k, a in pdata.items() if k]
        raise ValueError(f"Velocity field not found. Available point data fields: {avail}\n"
                         f"Specify velocity_field_name explicitly if using non-standard field names.")

    def load_single_timestep(self, time_idx: int) -> np.ndarray:
        if not 0 <= time_idx < len(self.time_files):
            raise IndexError(f"Time index {time_idx} out of range [0, {len(self.time_files) - 1}]")
        if time_idx in self.velocity_cache:
            return self.velocity_cache[time_idx]
        first = self.grid_points is None
        want = None if self.velocity_field_name is None else [self.velocity_field_name]
        d = read_vtk_xml(self.time_files[time_idx], geometry=first, names=want)
        if first:
            self.grid_points = np.ascontiguousarray(d["points"], dtype=F32)
            self._cells = d["cells"]
        name = self._field_name(d["point_data"])
        if name not in d["point_data"]:
            raise ValueError(f"Velocity field '{name}' not found in {self.time_files[time_idx]}")
        if d["point_data"][name] is None:          # decoded lazily for the chosen name
            d = read_vtk_xml(self.time_files[time_idx], geometry=False, names=[name])
        v = _velocity3(d["point_data"][name])
        if len(v) != len(self.grid_points):
            raise ValueError(f"Velocity field size mismatch in {self.time_files[time_idx]}: "
                             f"expected {len(self.grid_points)}, got {len(v)}")
        self.velocity_cache[time_idx] = v
        while len(self.velocity_cache) > self.cache_size_limit:
            self.velocity_cache.pop(next(iter(self.velocity_cache)))
        return v

    def __getitem__(self, time_idx: int) -> np.ndarray:
        return self.load_single_timestep(time_idx)

    def load_time_series(self, start_idx: int = 0, end_idx: Optional[int] = None) -> Dict[str, Any]:
        end = len(self.time_files) if end_idx is None else min(end_idx, len(self.time_files))
        if end - start_idx <= 0:
            raise ValueError(f"Invalid time range: [{start_idx}, {end})")
        first = self.load_single_timestep(start_idx)
        data = np.empty((end - start_idx, len(first), 3), dtype=F32)
        for k, i in enumerate(range(start_idx, end)):
            data[k] = self.load_single_timestep(i)
        return {"velocity_data": data, "positions": self.grid_points,
                "times": np.arange(start_idx, end, dtype=F32), "source": "vtk_unstructured_series",
                "file_pattern": self.file_pattern, "velocity_field_name": self.velocity_field_name}

    def tetrahedra(self) -> np.ndarray:
        """(M, 4) int32 vertex ids of the VTK_TETRA cells of the first file."""
        if self.grid_points is None:
            self.load_single_timestep(0)
        c = self._cells
        if not c:
            return np.zeros((0, 4), dtype=np.int32)
        types = np.asarray(c["types"])
        offs = np.asarray(c["offsets"], dtype=np.int64)
        conn = np.asarray(c["connectivity"], dtype=np.int64)
        starts = np.concatenate([[0], offs[:-1]])
        sel = (types == VTK_TETRA) & (offs - starts == 4)
        idx = starts[sel][:, None] + np.arange(4)[None, :]
        return conn[idx].astype(np.int32)

    def get_bounds(self) -> Tuple[float, ...]:
        if self.grid_points is None:
            self.load_single_timestep(0)
        lo, hi = self.grid_points.min(axis=0), self.grid_points.max(axis=0)
        return tuple(float(v) for v in (*lo, *hi))

    def get_grid_info(self) -> Dict[str, Any]:
        """The reference's keys (vtk_reader.py:773-788); no spatial index is
        built (nothing here queries the nodes by position)."""
        if self.grid_points is None:
            self.load_single_timestep(0)
        try:
            import psutil
            mem = psutil.Process().memory_info().rss / 1024 ** 3
        except ImportError:
            mem = 0.0
        return {"grid_points": self.grid_points, "n_points": int(len(self.grid_points)),
                "n_timesteps": len(self.time_files), "bounds": self.get_bounds(), "time_files": self.time_files,
                "velocity_field_name": self.velocity_field_name, "cache_size": len(self.velocity_cache),
                "memory_usage_gb": mem, "has_spatial_index": False}


def open_vtk_time_series(file_pattern: str, max_time_steps: Optional[int] = None,
                         velocity_field_name: Optional[str] = None, validate_files: bool = True,
                         **kwargs) -> Dict[str, Any]:
    """vtk_reader.py:944-988: the whole series in JAXTrace format."""
    reader = VTKUnstructuredTimeSeriesReader(file_pattern, max_time_steps=max_time_steps,
                                             velocity_field_name=velocity_field_name, **kwargs)
    return reader.load_time_series()


def _write_xml(path: str, kind: str, counts: Dict[str, int], sections: List[Tuple[str, List[Tuple[str, np.ndarray]]]],
               encoding: str, compress: bool, header: str) -> None:
    """One-piece VTK XML file of type ``kind`` (UnstructuredGrid or
    PolyData): ``sections`` in file order, each a list of (name, array) with
    (M,) or (M,C) arrays; a section name may carry attributes
    ('PointData Scalars="Time"')."""
    hdt = np.dtype(np.uint64 if header == "UInt64" else np.uint32).newbyteorder("<")

    def blob(a: np.ndarray) -> bytes:
        data = np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<")).tobytes()
        if not compress:
            return np.array([len(data)], dtype=hdt).tobytes() + data
        comp = zlib.compress(data)
        return np.array([1, len(data), len(data), len(comp)], dtype=hdt).tobytes() + comp

    appended = bytearray()
    body = []
    for sec, arrays in sections:
        parts = []
        for name, a in arrays:
            a = np.ascontiguousarray(a)
            nc = a.shape[1] if a.ndim > 1 else 1
            attrs = f'type="{_NAMES[np.dtype(a.dtype).newbyteorder("=")]}" Name="{name}" NumberOfComponents="{nc}"'
            if encoding == "ascii":
                text = " ".join(repr(x) if a.dtype.kind == "f" else str(x) for x in a.reshape(-1).tolist())
                parts.append(f'<DataArray {attrs} format="ascii">{text}</DataArray>')
            elif encoding == "binary":
                b = blob(a)
                if compress:
                    hs = hdt.itemsize * 4
                    text = base64.b64encode(b[:hs]).decode() + base64.b64encode(b[hs:]).decode()
                else:
                    text = base64.b64encode(b).decode()
                parts.append(f'<DataArray {attrs} format="binary">{text}</DataArray>')
            else:
                parts.append(f'<DataArray {attrs} format="appended" offset="{len(appended)}"/>')
                appended += blob(a)
        body.append(f'<{sec}>{"".join(parts)}</{sec.split()[0]}>\n')
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    piece = " ".join(f'{k}="{v}"' for k, v in counts.items())
    head = (f'<?xml version="1.0"?>\n<VTKFile type="{kind}" version="1.0" byte_order="LittleEndian" '
            f'header_type="{header}"{comp}>\n<{kind}>\n<Piece {piece}>\n{"".join(body)}</Piece>\n</{kind}>\n')
    with open(path, "wb") as fh:
        fh.write(head.encode())
        if encoding == "appended":
            fh.write(b'<AppendedData encoding="raw">\n_')
            fh.write(bytes(appended))
            fh.write(b"\n</AppendedData>\n")
        fh.write(b"</VTKFile>\n")


def write_vtu(path: str, points: np.ndarray, tets: Optional[np.ndarray] = None,
              point_data: Optional[Dict[str, np.ndarray]] = None, encoding: str = "appended",
              compress: bool = False, header: str = "UInt64", vertices: bool = False) -> None:
    """Write an UnstructuredGrid .vtu with point data: tetrahedra ``tets``,
    or with ``vertices`` one VTK_VERTEX cell per point.
    encoding: "appended" (raw), "binary" (base64) or "ascii"."""
    pts = np.ascontiguousarray(points, dtype=F32).reshape(-1, 3)
    if vertices:
        conn = np.arange(len(pts), dtype=np.int64)
        offs = np.arange(1, len(pts) + 1, dtype=np.int64)
        types = np.full(len(pts), VTK_VERTEX, dtype=np.uint8)
    else:
        t4 = np.zeros((0, 4), np.int64) if tets is None else np.asarray(tets, dtype=np.int64).reshape(-1, 4)
        conn, offs = t4.reshape(-1), 4 * np.arange(1, len(t4) + 1, dtype=np.int64)
        types = np.full(len(t4), VTK_TETRA, dtype=np.uint8)
    pdata = [(k, np.asarray(v).reshape(len(pts), -1) if np.ndim(v) > 1 else np.asarray(v))
             for k, v in (point_data or {}).items()]
    _write_xml(path, "UnstructuredGrid", {"NumberOfPoints": len(pts), "NumberOfCells": len(types)},
               [("PointData", pdata), ("Points", [("Points", pts)]),
                ("Cells", [("connectivity", conn), ("offsets", offs), ("types", types)])],
               encoding, compress, header)


def write_vtp(path: str, points: np.ndarray, verts: Optional[Tuple[np.ndarray, np.ndarray]] = None,
              lines: Optional[Tuple[np.ndarray, np.ndarray]] = None,
              point_data: Optional[Dict[str, np.ndarray]] = None, cell_data: Optional[Dict[str, np.ndarray]] = None,
              encoding: str = "appended", compress: bool = False, header: str = "UInt64",
              point_scalars: Optional[str] = None, cell_scalars: Optional[str] = None) -> None:
    """Write a PolyData .vtp: ``verts`` and ``lines`` are (connectivity,
    offsets) pairs (offsets = running end of each cell's point list);
    ``cell_data`` arrays run over the verts and then the lines;
    ``point_scalars`` / ``cell_scalars`` name the active scalar arrays."""
    pts = np.ascontiguousarray(points, dtype=F32).reshape(-1, 3)
    empty = (np.zeros(0, np.int64), np.zeros(0, np.int64))
    vc, vo = [np.asarray(a, dtype=np.int64) for a in (verts or empty)]
    lc, lo = [np.asarray(a, dtype=np.int64) for a in (lines or empty)]
    pdata = [(k, np.asarray(v)) for k, v in (point_data or {}).items()]
    cdata = [(k, np.asarray(v)) for k, v in (cell_data or {}).items()]
    _write_xml(path, "PolyData", {"NumberOfPoints": len(pts), "NumberOfVerts": len(vo), "NumberOfLines": len(lo),
                                  "NumberOfStrips": 0, "NumberOfPolys": 0},
               [("PointData" + (f' Scalars="{point_scalars}"' if point_scalars else ""), pdata),
                ("CellData" + (f' Scalars="{cell_scalars}"' if cell_scalars else ""), cdata), ("Points", [("Points", pts)]),
                ("Verts", [("connectivity", vc), ("offsets", vo)]), ("Lines", [("connectivity", lc), ("offsets", lo)])],
               encoding, compress, header)


def write_pvtu(path: str, sources: List[str], point_arrays: Dict[str, Tuple[str, int]]) -> None:
    """A .pvtu naming existing .vtu pieces (paths relative to the .pvtu)."""
    pd = "".join(f'<PDataArray type="{t}" Name="{n}" NumberOfComponents="{c}"/>' for n, (t, c) in point_arrays.items())
    pieces = "".join(f'<Piece Source="{s}"/>' for s in sources)
    with open(path, "w") as fh:
        fh.write(f'<?xml version="1.0"?>\n<VTKFile type="PUnstructuredGrid" version="1.0" byte_order="LittleEndian">\n'
                 f'<PUnstructuredGrid GhostLevel="0"><PPointData>{pd}</PPointData>'
                 f'<PPoints><PDataArray type="Float32" NumberOfComponents="3"/></PPoints>{pieces}'
                 f'</PUnstructuredGrid>\n</VTKFile>\n')


class VTKTrajectoryWriter:
    """Trajectory files for ParaView (io/vtk_writer.py:58-300), written
    without the VTK library as zlib-compressed PolyData .vtp files."""

    def __init__(self, output_dir: str):
        self.output_dir = os.fspath(output_dir)
        os.makedirs(self.output_dir, exist_ok=True)

    def write_trajectory_points(self, trajectory_positions: np.ndarray, times: np.ndarray,
                                filename: str = "particle_trajectories.vtp",
                                particle_data: Optional[Dict[str, np.ndarray]] = None,
                                time_subset: Optional[slice] = None) -> str:
        """Every (row, particle) position as a vertex (vtk_writer.py:84-197):
        point arrays Time, ParticleID and TimeStep (float32), plus each
        ``particle_data`` array of shape (N,) (repeated per row) or (T, N);
        other shapes are skipped with a warning.  ``time_subset`` slices
        the rows, and the (T, N) arrays with them."""
        pos = np.asarray(trajectory_positions, dtype=F32)
        times = np.asarray(times)
        T_all, N = pos.shape[0], pos.shape[1]
        if time_subset is not None:
            pos, times = pos[time_subset], times[time_subset]
        T = pos.shape[0]
        pts = pos.reshape(-1, 3)
        if pts.ndim != 2 or pts.shape[1] != 3:
            raise ValueError(f"Positions must have 3 coordinates, got shape {pos.shape}")
        n = T * N
        pdata = {"Time": np.repeat(times, N).astype(F32),
                 "ParticleID": np.tile(np.arange(N, dtype=F32), T),
                 "TimeStep": np.repeat(np.arange(T, dtype=F32), N)}
        for name, data in (particle_data or {}).items():
            d = np.asarray(data, dtype=F32)
            if time_subset is not None and d.ndim == 2 and d.shape[0] == T_all:
                d = d[time_subset]
            if d.ndim == 1 and len(d) == N:
                pdata[name] = np.tile(d, T)
            elif d.ndim == 2 and d.shape == (T, N):
                pdata[name] = d.ravel()
            else:
                warnings.warn(f"Skipping data '{name}' - incompatible shape {d.shape}")
        path = os.path.join(self.output_dir, filename)
        write_vtp(path, pts, verts=(np.arange(n), np.arange(1, n + 1)), point_data=pdata, compress=True,
                  point_scalars="Time")
        return path

    def write_trajectory_lines(self, trajectory_positions: np.ndarray, times: np.ndarray,
                               filename: str = "particle_paths.vtp", max_particles: Optional[int] = None,
                               particle_subset: Optional[np.ndarray] = None) -> str:
        """One polyline per particle through its rows (vtk_writer.py:199-300):
        points row-major over the selected particles, point arrays Time and
        ParticleID (float32), cell array PathLength (float32 sum of the
        segment lengths).  ``max_particles`` keeps linspace(0, N-1, m)
        particles; ``particle_subset`` names them."""
        pos = np.asarray(trajectory_positions, dtype=F32)
        T, N = pos.shape[0], pos.shape[1]
        if particle_subset is not None:
            idx = np.asarray(particle_subset)
        elif max_particles is not None and N > max_particles:
            idx = np.linspace(0, N - 1, max_particles, dtype=int)
        else:
            idx = np.arange(N)
        ns = len(idx)
        sel = pos[:, idx, :]
        conn = (np.arange(T, dtype=np.int64)[None, :] * ns + np.arange(ns, dtype=np.int64)[:, None]).ravel()
        offs = T * np.arange(1, ns + 1, dtype=np.int64)
        # per particle, a contiguous float32 sum of its segment lengths
        seg = np.linalg.norm(np.diff(sel, axis=0), axis=2)
        plen = np.sum(np.ascontiguousarray(seg.T), axis=1).astype(F32) if T > 1 else np.zeros(ns, F32)
        path = os.path.join(self.output_dir, filename)
        write_vtp(path, sel.reshape(-1, 3), lines=(conn, offs),
                  point_data={"Time": np.repeat(np.asarray(times), ns).astype(F32),
                              "ParticleID": np.tile(idx.astype(F32), T)},
                  cell_data={"PathLength": plen}, compress=True, point_scalars="Time", cell_scalars="PathLength")
        return path


def write_pvd(path: str, files: List[str], times) -> None:
    """A .pvd collection of ``files`` (relative to the .pvd) at ``times``
    (io/vtk_writer.py:609-626)."""
    with open(path, "w") as fh:
        fh.write('<?xml version="1.0"?>\n<VTKFile type="Collection" version="0.1">\n  <Collection>\n')
        for f, t in zip(files, times):
            fh.write(f'    <DataSet timestep="{float(t):.6f}" file="{f}"/>\n')
        fh.write("  </Collection>\n</VTKFile>\n")


class VTKTrajectorySeries:
    """A ``TrackerOptions.row_sink`` that streams a trajectory to disk while
    it is tracked: each row as ``{prefix}_{row:04d}.vtu`` (one vertex per
    particle; point arrays Time, ParticleID and, when velocities are
    recorded, Velocity and Speed -- the per-row content of
    Trajectory.export_to_vtk) and, on ``close()``, the ``{prefix}.pvd``
    collection over them."""

    def __init__(self, output_dir: str, prefix: str = "particles", encoding: str = "appended",
                 compress: bool = False):
        self.output_dir = os.fspath(output_dir)
        os.makedirs(self.output_dir, exist_ok=True)
        self.prefix, self.encoding, self.compress = prefix, encoding, compress
        self.files: List[str] = []
        self.times: List[float] = []

    def __call__(self, first_row: int, positions: np.ndarray, velocities: Optional[np.ndarray],
                 row_times: np.ndarray) -> None:
        for i in range(len(positions)):
            n = positions.shape[1]
            pdata = {"Time": np.full(n, row_times[i], dtype=F32), "ParticleID": np.arange(n, dtype=np.int32)}
            if velocities is not None:
                v = np.asarray(velocities[i], dtype=F32)
                pdata["Velocity"] = v
                pdata["Speed"] = np.linalg.norm(v, axis=1).astype(F32)
            name = f"{self.prefix}_{first_row + i:04d}.vtu"
            write_vtu(os.path.join(self.output_dir, name), positions[i], point_data=pdata, encoding=self.encoding,
                      compress=self.compress, vertices=True)
            self.files.append(name)
            self.times.append(float(row_times[i]))

    def close(self) -> str:
        path = os.path.join(self.output_dir, f"{self.prefix}.pvd")
        write_pvd(path, self.files, self.times)
        return path


def open_dataset(path_spec, format_type: Optional[str] = None, **kwargs):
    """io/registry.py:252-343 for the formats this package reads: VTK
    (.vtu/.pvtu/.vtk, a pattern or a list of files) opens a
    VTKUnstructuredTimeSeriesReader; HDF5 reports its backend unavailable
    (h5py is not installed)."""
    files = sorted(glob.glob(os.path.expanduser(path_spec))) if isinstance(path_spec, str) else list(path_spec)
    files = [f for f in files if os.path.exists(f)]
    if not files:
        raise FileNotFoundError(f"No files found matching: {path_spec}")
    ext = os.path.splitext(files[0].lower())[1]
    if format_type is None:
        format_type = {".vtu": "vtk", ".pvtu": "vtk", ".vtk": "vtk", ".vtp": "vtk", ".h5": "hdf5", ".hdf5": "hdf5",
                       ".hdf": "hdf5"}.get(ext)
        if format_type is None:
            raise ValueError(f"Unknown file format '{ext}' for file: {files[0]}")
    if format_type == "hdf5":
        raise ImportError("HDF5 backend not available. Install required package for HDF5 (h5py)")
    if format_type != "vtk":
        raise ValueError(f"Unsupported format: {format_type}")
    return VTKUnstructuredTimeSeriesReader(path_spec if isinstance(path_spec, str) else files, **kwargs)


def create_time_series_from_vtk_files(file_pattern: str, velocity_field_name: Optional[str] = "velocity",
                                      max_time_steps: Optional[int] = None, **kwargs):
    """TimeSeriesField over a VTK time series (fields/time_series.py:606-628);
    a velocity name absent from the files falls back to detection."""
    from .fields import TimeSeriesField
    reader = VTKUnstructuredTimeSeriesReader(file_pattern, max_time_steps=max_time_steps)
    first = read_vtk_xml(reader.time_files[0], geometry=False, names=[])
    if velocity_field_name is not None and velocity_field_name in first["point_data"]:
        reader.velocity_field_name = velocity_field_name
    d = reader.load_time_series()
    return TimeSeriesField(data=d["velocity_data"], times=d["times"], positions=d["positions"],
                           _source_info=d.get("source_info", {}), **kwargs)


def create_field_from_vtk(file_pattern: str, field_type: str = "auto", **kwargs):
    """fields/__init__.py:114-207 for unstructured VTK data: several files
    (or field_type "time_series") give a time series, one .vtu/.pvtu/.vtk
    file a single-snapshot nearest-node field; structured image/grid files
    (.vti/.vts/.vtr) are not read here."""
    if os.path.isdir(file_pattern):
        files = sorted(f for ext in ("*.vtu", "*.pvtu", "*.vtk", "*.vti", "*.vts", "*.vtr")
                       for f in glob.glob(os.path.join(file_pattern, ext)))
        # the pattern of the extension the reader will take: .pvtu, else .vtu, else legacy .vtk
        exts = {os.path.splitext(f)[1].lower() for f in files}
        ext = next((e for e in (".pvtu", ".vtu", ".vtk") if e in exts), ".vtu")
        pattern = os.path.join(file_pattern, "*" + ext)
    else:
        files = sorted(glob.glob(os.path.expanduser(file_pattern)))
        pattern = file_pattern
    if not files:
        raise FileNotFoundError(f"No VTK files found: {file_pattern}")
    if field_type == "auto":
        if len(files) > 1:
            field_type = "time_series"
        elif files[0].lower().endswith((".vti", ".vts", ".vtr")):
            field_type = "structured"
        else:
            field_type = "unstructured"
    if field_type == "time_series":
        return create_time_series_from_vtk_files(pattern, **kwargs)
    if field_type == "structured":
        raise NotImplementedError("structured VTK files (.vti/.vts/.vtr) are not read; use "
                                  "StructuredTimeSeriesField with the grid arrays")
    if field_type == "unstructured":
        from .fields import TimeSeriesField
        d = read_vtk_xml(files[0])
        name = next((n for n in VELOCITY_NAMES if n in d["point_data"]), None)
        if name is None:
            raise ValueError(f"{files[0]}: no velocity array among {list(d['point_data'])}")
        v = _velocity3(np.asarray(d["point_data"][name]))
        return TimeSeriesField(data=v[None], times=np.zeros(1, F32), positions=d["points"], **kwargs)
    raise ValueError(f"Unknown field type: {field_type}")
