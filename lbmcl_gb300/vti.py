"""VTK ImageData (.vti) reading and writing without VTK.

* `read_vti` reads the encodings this project meets: the ASCII files the
  lbmcl host writes (lbmcl.hpp:261-334), the raw appended files of its
  `--format binary`, and the appended, base64, zlib compressed files of the
  reference's golden data (written by Sailfish).
* `write_vti_binary` writes the same ImageData with raw appended data,
  optionally zlib compressed in VTK's block format (vtkZLibDataCompressor).
* `read_f_raw` reads an f_<it>.raw dump (the f buffer in the CSoA layout of
  the run's stride) back into [19, dim^3] site-major arrays.
* `write_vti_ascii` writes the reference's ASCII layout byte for byte
  (lbmcl.hpp:284-331): interior points [1, dim-2]^3, `%.16e`-style scientific
  numbers each followed by a space, one line per (y, z) row.
* `compare` computes the two figures the reference's verify.py prints for one
  file pair (verify.py:44-60): mean squared error and max absolute error of
  rho and of v, NaN mapped to 0.
"""
from __future__ import annotations

import base64
import re
import zlib

import numpy as np

_DT = {"Float32": np.float32, "Float64": np.float64, "UInt32": np.uint32, "UInt64": np.uint64,
       "Int32": np.int32, "Int64": np.int64, "UInt8": np.uint8}


def _attr(tag: str, name: str):
    m = re.search(r'\b%s="([^"]*)"' % name, tag)
    return m.group(1) if m else None


def _decode_appended_b64(text: str, start: int, dtype, header_t, compressed: bool) -> np.ndarray:
    hsz = np.dtype(header_t).itemsize
    if not compressed:
        nch = 4 * ((hsz + 2) // 3)
        raw = base64.b64decode(text[start:start + nch])
        nbytes = int(np.frombuffer(raw[:hsz], header_t)[0])
        total = 4 * ((hsz + nbytes + 2) // 3)
        raw = base64.b64decode(text[start:start + total])
        return np.frombuffer(raw[hsz:hsz + nbytes], dtype).copy()
    first = base64.b64decode(text[start:start + 4 * ((hsz + 2) // 3) + 4])
    nblocks = int(np.frombuffer(first[:hsz], header_t)[0])
    hbytes = (3 + nblocks) * hsz
    hch = 4 * ((hbytes + 2) // 3)
    hdr = np.frombuffer(base64.b64decode(text[start:start + hch])[:hbytes], header_t).astype(np.int64)
    _, bsize, last = hdr[0], int(hdr[1]), int(hdr[2])
    csizes = [int(c) for c in hdr[3:3 + nblocks]]
    total = sum(csizes)
    dch = 4 * ((total + 2) // 3)
    data = base64.b64decode(text[start + hch:start + hch + dch])
    out, pos = [], 0
    for k, cs in enumerate(csizes):
        blk = zlib.decompress(data[pos:pos + cs])
        want = last if (k == nblocks - 1 and last) else bsize
        assert len(blk) == want, "corrupt zlib block"
        out.append(blk)
        pos += cs
    return np.frombuffer(b"".join(out), dtype).copy()


def _decode_appended_raw(data: bytes, start: int, dtype, header_t, compressed: bool) -> np.ndarray:
    hsz = np.dtype(header_t).itemsize
    if not compressed:
        nbytes = int(np.frombuffer(data, header_t, 1, start)[0])
        return np.frombuffer(data, dtype, nbytes // np.dtype(dtype).itemsize, start + hsz).copy()
    nblocks = int(np.frombuffer(data, header_t, 1, start)[0])
    hdr = np.frombuffer(data, header_t, 3 + nblocks, start).astype(np.int64)
    bsize, last = int(hdr[1]), int(hdr[2])
    pos = start + (3 + nblocks) * hsz
    out = []
    for k, cs in enumerate(int(c) for c in hdr[3:]):
        blk = zlib.decompress(data[pos:pos + cs])
        want = last if (k == nblocks - 1 and last) else bsize
        assert len(blk) == want, "corrupt zlib block"
        out.append(blk)
        pos += cs
    return np.frombuffer(b"".join(out), dtype).copy()


def read_vti(path: str) -> dict:
    """Return {"extent": (x0,x1,y0,y1,z0,z1), name: array, ...}.  Vector arrays
    come back as [npoints, ncomp]."""
    with open(path, "rb") as fh:
        data = fh.read()
    # the XML part is ASCII; raw appended bytes follow the '_' of AppendedData
    text = data.decode("latin-1")
    head = re.search(r"<VTKFile[^>]*>", text).group(0)
    header_t = _DT.get(_attr(head, "header_type") or "UInt32", np.uint32)
    compressed = _attr(head, "compressor") is not None
    img = re.search(r"<ImageData[^>]*>", text).group(0)
    ext = tuple(int(v) for v in _attr(img, "WholeExtent").split())
    out = {"extent": ext}
    app = re.search(r"<AppendedData[^>]*>\s*_", text)
    app_start = app.end() if app else None
    raw = app is not None and _attr(app.group(0), "encoding") == "raw"
    for m in re.finditer(r"<DataArray([^>]*)>(.*?)</DataArray>|<DataArray([^>]*)/>", text, re.S):
        tag = m.group(1) or m.group(3)
        name = _attr(tag, "Name")
        dtype = _DT[_attr(tag, "type")]
        ncomp = int(_attr(tag, "NumberOfComponents") or 1)
        fmt = _attr(tag, "format")
        if fmt == "ascii":
            arr = np.array(m.group(2).split(), dtype=np.float64).astype(dtype)
        elif fmt == "appended":
            off = int(_attr(tag, "offset"))
            if raw:
                arr = _decode_appended_raw(data, app_start + off, dtype, header_t, compressed)
            else:
                arr = _decode_appended_b64(text, app_start + off, dtype, header_t, compressed)
        else:
            raise ValueError(f"unsupported DataArray format {fmt!r}")
        out[name] = arr.reshape(-1, ncomp) if ncomp > 1 else arr
    return out


def _fmt(v: float) -> str:
    """std::scientific with setprecision(16) (lbmcl.hpp:303, 319-321)."""
    return "%.16e" % v


def write_vti_ascii(path: str, dim: int, rho: np.ndarray, u: np.ndarray) -> None:
    """ASCII VTI of the interior [1, dim-2]^3 in the reference's layout.
    rho: dim^3, u: 3*dim^3 planar (lbmcl.hpp:19-23)."""
    n = dim ** 3
    ext = dim - 3
    tname = "Float32" if rho.dtype == np.float32 else "Float64"
    r = rho.reshape(dim, dim, dim)[1:dim - 1, 1:dim - 1, 1:dim - 1]
    uu = u.reshape(3, dim, dim, dim)[:, 1:dim - 1, 1:dim - 1, 1:dim - 1]
    lines = [
        '<?xml version="1.0"?>\n',
        '<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian" header_type="UInt64">\n',
        f'  <ImageData WholeExtent="0 {ext} 0 {ext} 0 {ext}" Origin="0 0 0" Spacing="1 1 1">\n',
        f'    <Piece Extent="0 {ext} 0 {ext} 0 {ext}">\n',
        '      <PointData Scalars="rho">\n',
        f'        <DataArray type="{tname}" Name="rho" NumberOfComponents="1" format="ascii">\n',
    ]
    del n
    rr = r.astype(np.float64)
    for z in range(dim - 2):
        for y in range(dim - 2):
            lines.append("".join(_fmt(v) + " " for v in rr[z, y]) + "\n")
    lines.append("        </DataArray>\n")
    lines.append(f'        <DataArray type="{tname}" Name="v" NumberOfComponents="3" format="ascii">\n')
    ud = uu.astype(np.float64)
    for z in range(dim - 2):
        for y in range(dim - 2):
            lines.append("".join(_fmt(ud[0, z, y, x]) + " " + _fmt(ud[1, z, y, x]) + " " + _fmt(ud[2, z, y, x]) + " "
                                 for x in range(dim - 2)) + "\n")
    lines += ["        </DataArray>\n", "      </PointData>\n", "    </Piece>\n", "  </ImageData>\n", "</VTKFile>\n"]
    with open(path, "w") as fh:
        fh.write("".join(lines))


def _zlib_blocks(payload: bytes, block: int, level: int) -> bytes:
    """VTK's vtkZLibDataCompressor layout with a UInt64 header: [nblocks,
    block size, size of the last block, compressed sizes...] then the blocks."""
    chunks = [payload[i:i + block] for i in range(0, len(payload), block)] or [b""]
    comp = [zlib.compress(c, level) for c in chunks]
    last = len(chunks[-1]) if len(chunks[-1]) != block else 0
    hdr = np.array([len(chunks), block, last] + [len(c) for c in comp], np.uint64)
    return hdr.tobytes() + b"".join(comp)


def write_vti_binary(path: str, dim: int, rho: np.ndarray, u: np.ndarray, compress: bool = False,
                     level: int = 6, block: int = 1 << 20) -> None:
    """The interior [1, dim-2]^3 ImageData of write_vti_ascii, with raw
    appended data (UInt64 headers; rho, then v interleaved).  compress=True
    stores each array zlib-compressed in VTK's block format."""
    f = interior_fields(dim, rho, u)
    tname = "Float32" if rho.dtype == np.float32 else "Float64"
    ext = dim - 3
    blobs = []
    for name in ("rho", "v"):
        payload = np.ascontiguousarray(f[name]).tobytes()
        blobs.append(_zlib_blocks(payload, block, level) if compress
                     else np.array([len(payload)], np.uint64).tobytes() + payload)
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    head = (
        '<?xml version="1.0"?>\n'
        f'<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian" header_type="UInt64"{comp}>\n'
        f'  <ImageData WholeExtent="0 {ext} 0 {ext} 0 {ext}" Origin="0 0 0" Spacing="1 1 1">\n'
        f'    <Piece Extent="0 {ext} 0 {ext} 0 {ext}">\n'
        '      <PointData Scalars="rho">\n'
        f'        <DataArray type="{tname}" Name="rho" NumberOfComponents="1" format="appended" offset="0"/>\n'
        f'        <DataArray type="{tname}" Name="v" NumberOfComponents="3" format="appended" '
        f'offset="{len(blobs[0])}"/>\n'
        '      </PointData>\n'
        '    </Piece>\n'
        '  </ImageData>\n'
        '  <AppendedData encoding="raw">\n   _')
    with open(path, "wb") as fh:
        fh.write(head.encode("ascii"))
        for b in blobs:
            fh.write(b)
        fh.write(b"\n  </AppendedData>\n</VTKFile>\n")


def read_f_raw(path: str, dim: int, stride: int, dtype=np.float32) -> np.ndarray:
    """An f_<it>.raw dump (19 * dim^3 values in the CSoA layout of `stride`,
    lbmcl.hpp:19-23) as a [19, dim^3] array indexed [q, site]."""
    n = dim ** 3
    f = np.fromfile(path, dtype)
    if f.size != 19 * n:
        raise ValueError(f"{path}: {f.size} values, expected {19 * n}")
    if stride <= 0 or stride >= n:
        return f.reshape(19, n).copy()
    return f.reshape(n // stride, 19, stride).transpose(1, 0, 2).reshape(19, n).copy()


def compare(target: dict, prediction: dict) -> dict:
    """verify.py:44-60 for one pair: MSE and max-abs of rho and v, NaN -> 0.
    MSE of v averages over points and components, as sklearn's
    mean_squared_error does for 2-D input."""
    tr = np.nan_to_num(np.asarray(target["rho"], np.float64))
    pr = np.nan_to_num(np.asarray(prediction["rho"], np.float64))
    tv = np.nan_to_num(np.asarray(target["v"], np.float64))
    pv = np.nan_to_num(np.asarray(prediction["v"], np.float64))
    return {
        "mse_rho": float(np.mean((tr - pr) ** 2)),
        "mse_v": float(np.mean((tv - pv) ** 2)),
        "mae_rho": float(np.max(np.abs(tr - pr))),
        "mae_v": float(np.max(np.abs(tv - pv))),
    }


def interior_fields(dim: int, rho: np.ndarray, u: np.ndarray) -> dict:
    """rho/u arrays (dim^3, 3*dim^3) -> the point arrays a VTI of the interior holds."""
    r = rho.reshape(dim, dim, dim)[1:dim - 1, 1:dim - 1, 1:dim - 1].reshape(-1)
    uu = u.reshape(3, dim, dim, dim)[:, 1:dim - 1, 1:dim - 1, 1:dim - 1].reshape(3, -1).T
    return {"rho": r, "v": np.ascontiguousarray(uu)}

