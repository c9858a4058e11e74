"""Dose-map utilities of the reference (pyvoxeldosimetry/core/utils.py) on the
dose the GPU path produces: the dose-volume histogram (GPU), the NIfTI dose-map
format (host) and spacing resampling (GPU).
"""
from __future__ import annotations

import ctypes as C
import gzip as _gzip
import json as _json
import struct as _struct
from pathlib import Path as _Path
from typing import Tuple

import numpy as np
import torch

from .. import _native as N
from ..conv import _require_cuda


def _dose_on_device(x, device):
    """(CUDA tensor, PVD_DTYPE, numpy type): float32 / float64 kept as they are (the
    histogram's arithmetic runs in the dose's own type, as numpy's does), any other
    type promoted to float64 as numpy's bin type would be."""
    if isinstance(x, torch.Tensor):
        t = x if x.dtype in (torch.float32, torch.float64) else x.double()
        t = t.to(device).contiguous()
    else:
        a = np.asarray(x)
        if a.dtype not in (np.float32, np.float64):
            a = a.astype(np.float64)
        t = torch.from_numpy(np.ascontiguousarray(a)).to(device)
    if t.dtype == torch.float32:
        return t, N.PVD_DTYPE_F32, np.float32
    return t, N.PVD_DTYPE_F64, np.float64


def _mask_on_device(m, device):
    """(CUDA tensor, PVD_DTYPE): bool / uint8 as bytes, float32 as is (voxels with
    mask > 0 count), any other type reduced to (mask > 0) bytes."""
    if isinstance(m, torch.Tensor):
        if m.dtype == torch.bool:
            t = m.to(torch.uint8)
        elif m.dtype in (torch.uint8, torch.float32):
            t = m
        else:
            t = (m > 0).to(torch.uint8)
        t = t.to(device).contiguous()
    else:
        a = np.asarray(m)
        if a.dtype == np.bool_:
            a = a.view(np.uint8)
        elif a.dtype not in (np.uint8, np.float32):
            a = (a > 0).view(np.uint8)
        t = torch.from_numpy(np.ascontiguousarray(a)).to(device)
    return t, (N.PVD_DTYPE_F32 if t.dtype == torch.float32 else N.PVD_DTYPE_U8)


def calculate_dvh(dose_map, roi_mask, bins: int = 1000, device=None) -> Tuple[np.ndarray, np.ndarray]:
    """Cumulative dose-volume histogram of the doses inside ``roi_mask > 0``.

    Same contract as the reference (core/utils.py:233-262): bins uniform between
    the ROI's minimum and maximum dose (np.histogram with an integer bin count),
    returns ``(edges[1:], 1 - cumsum(hist) / n)`` as numpy arrays; raises
    ValueError for mismatched shapes, an empty ROI or a non-finite ROI dose.
    ``dose_map`` / ``roi_mask`` may be numpy arrays or torch tensors (CUDA ones are
    used in place).  The ROI statistics and the counts are computed on the GPU
    with numpy's arithmetic, so the result equals the reference's exactly.
    """
    if tuple(dose_map.shape) != tuple(roi_mask.shape):
        raise ValueError("Dose map and ROI mask must have same dimensions")
    if isinstance(bins, bool) or not isinstance(bins, (int, np.integer)):
        raise TypeError("bins must be an integer (the reference's calculate_dvh takes a bin count)")
    if bins < 1:
        raise ValueError("`bins` must be positive, when an integer")
    dev = _require_cuda(device)
    lib = N.load()
    bins = int(bins)
    with torch.cuda.device(dev):
        d, dt, np_t = _dose_on_device(dose_map, dev)
        m, mt = _mask_on_device(roi_mask, dev)
        if d.numel() == 0:
            raise ValueError("ROI mask is empty")
        # statistics, numpy's edges and the counts on the device; one copy back
        res = torch.empty(4 + bins, dtype=torch.int64, device=dev)
        edges_d = torch.empty(bins + 1, dtype=d.dtype, device=dev)
        N.check(lib.pvd_dvh(d.data_ptr(), dt, m.data_ptr(), mt, d.numel(), bins, edges_d.data_ptr(),
                            res.data_ptr(), torch.cuda.current_stream(dev).cuda_stream))
        host = res.cpu().numpy()
    count, nonfinite = int(host[2]), int(host[3])
    if count == 0:
        raise ValueError("ROI mask is empty")
    if nonfinite:
        raise ValueError("autodetected range of [nan, nan] is not finite")
    first, last = _key_values(host[:2].view(np.uint64), np_t)
    if first == last:
        first, last = first - 0.5, last + 0.5
    edges = np.linspace(first, last, bins + 1, endpoint=True, dtype=np_t)
    cum_dvh = 1.0 - np.cumsum(host[4:]) / count
    return edges[1:], cum_dvh


def _key_values(keys: np.ndarray, np_t):
    """Doses back from pvd_dvh's order-preserving keys (inverse of the device encoding)."""
    if np_t is np.float32:
        u = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        b = np.where(u & np.uint32(0x80000000), u & np.uint32(0x7FFFFFFF), ~u).astype(np.uint32)
        v = b.view(np.float32)
    else:
        sign = np.uint64(0x8000000000000000)
        b = np.where(keys & sign, keys & np.uint64(0x7FFFFFFFFFFFFFFF), ~keys).astype(np.uint64)
        v = b.view(np.float64)
    return np_t(v[0]), np_t(v[1])


# ---------------------------------------------------------------------------
# NIfTI-1 dose maps (core/utils.py:53-152).  The reference writes and reads them
# through nibabel; this is a self-contained writer/reader of the NIfTI-1
# single-file format (.nii, .nii.gz) with the same content: float32 data, first
# array axis fastest in the file, pixdim = voxel size, sform = the affine
# (code 2, "aligned"), the qform as the quaternion of the affine's rotation
# (code 0), descrip, and the metadata as JSON in an extension of code 44.
# ---------------------------------------------------------------------------
_NIFTI_HDR = 348
_DT_NUMPY = {2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64, 256: np.int8,
             512: np.uint16, 768: np.uint32, 1024: np.int64, 1280: np.uint64}


def _quatern_from_affine(affine: np.ndarray):
    """NIfTI-1 qform parameters (b, c, d, qfac) of the rotation in a 4x4 affine:
    columns normalised by the voxel sizes, a reflection moved into qfac = -1 by
    negating the third column, then the rotation matrix's unit quaternion
    (a >= 0), following the NIfTI-1 header specification."""
    m = np.asarray(affine, dtype=np.float64)[:3, :3].copy()
    zooms = np.sqrt((m * m).sum(axis=0))
    zooms[zooms == 0] = 1.0
    r = m / zooms
    qfac = 1.0
    if np.linalg.det(r) < 0:
        qfac = -1.0
        r[:, 2] = -r[:, 2]
    # orthonormalise (the nearest rotation) before taking the quaternion
    u, _, vt = np.linalg.svd(r)
    r = u @ vt
    tr = r[0, 0] + r[1, 1] + r[2, 2]
    if tr > 0.5:
        a = 0.5 * np.sqrt(1.0 + tr)
        b = 0.25 * (r[2, 1] - r[1, 2]) / a
        c = 0.25 * (r[0, 2] - r[2, 0]) / a
        d = 0.25 * (r[1, 0] - r[0, 1]) / a
    elif r[0, 0] >= r[1, 1] and r[0, 0] >= r[2, 2]:
        b = 0.5 * np.sqrt(1.0 + r[0, 0] - r[1, 1] - r[2, 2])
        a = 0.25 * (r[2, 1] - r[1, 2]) / b
        c = 0.25 * (r[0, 1] + r[1, 0]) / b
        d = 0.25 * (r[0, 2] + r[2, 0]) / b
    elif r[1, 1] >= r[2, 2]:
        c = 0.5 * np.sqrt(1.0 - r[0, 0] + r[1, 1] - r[2, 2])
        a = 0.25 * (r[0, 2] - r[2, 0]) / c
        b = 0.25 * (r[0, 1] + r[1, 0]) / c
        d = 0.25 * (r[1, 2] + r[2, 1]) / c
    else:
        d = 0.5 * np.sqrt(1.0 - r[0, 0] - r[1, 1] + r[2, 2])
        a = 0.25 * (r[1, 0] - r[0, 1]) / d
        b = 0.25 * (r[0, 2] + r[2, 0]) / d
        c = 0.25 * (r[1, 2] + r[2, 1]) / d
    if a < 0:
        b, c, d = -b, -c, -d
    return float(b), float(c), float(d), qfac


def _nifti_bytes(data: np.ndarray, voxel_size, affine: np.ndarray, descrip: str, extension: bytes) -> bytes:
    data = np.asarray(data, dtype=np.float32)
    if data.ndim < 1 or data.ndim > 7:
        raise ValueError("NIfTI-1 holds 1 to 7 dimensions")
    esize = 8 + len(extension)
    esize += (-esize) % 16
    vox_offset = _NIFTI_HDR + 4 + (esize if extension else 0)
    dim = [data.ndim] + list(data.shape) + [1] * (7 - data.ndim)
    pixdim = [0.0] * 8
    b, c, d, qfac = _quatern_from_affine(affine)
    pixdim[0] = qfac
    for i, v in enumerate(tuple(voxel_size)[: min(7, data.ndim)]):
        pixdim[1 + i] = float(v)
    aff = np.asarray(affine, dtype=np.float64)
    h = bytearray(_NIFTI_HDR)
    _struct.pack_into("<i", h, 0, _NIFTI_HDR)
    h[38] = ord("r")
    _struct.pack_into("<8h", h, 40, *dim)
    _struct.pack_into("<hhh", h, 68, 0, 16, 32)                 # intent_code, datatype FLOAT32, bitpix
    _struct.pack_into("<8f", h, 76, *pixdim)
    _struct.pack_into("<fff", h, 108, float(vox_offset), 1.0, 0.0)  # vox_offset, scl_slope, scl_inter
    h[123] = 2                                                   # xyzt_units: millimetres
    desc = descrip.encode("utf-8")[:79]
    h[148:148 + len(desc)] = desc
    _struct.pack_into("<hh", h, 252, 0, 2)                      # qform_code unknown, sform_code aligned
    _struct.pack_into("<6f", h, 256, b, c, d, *aff[:3, 3])
    _struct.pack_into("<12f", h, 280, *aff[0, :4], *aff[1, :4], *aff[2, :4])
    h[344:348] = b"n+1\x00"
    out = bytearray(h)
    out += bytes([1 if extension else 0, 0, 0, 0])
    if extension:
        out += _struct.pack("<ii", esize, 44) + extension + bytes(esize - 8 - len(extension))
    assert len(out) == vox_offset
    out += np.asarray(data, dtype="<f4").tobytes(order="F")
    return bytes(out)


def save_dose_map(filename, dose_map, voxel_size: Tuple[float, float, float], metadata: dict, affine=None) -> None:
    """Write a dose map as NIfTI-1 (core/utils.py:53-103): ``.nii`` or ``.nii.gz``
    (appended when the name has neither); default affine diag(voxel_size) with the
    volume centred on the origin; ``metadata`` is updated in place with the
    reference's fields (its fixed creation date and author, voxel size,
    dimensions, affine) and stored as JSON in an extension of code 44.
    ``dose_map`` may be a numpy array or a torch tensor (copied to the host)."""
    filename = str(filename)
    if not filename.endswith((".nii", ".nii.gz")):
        filename += ".nii.gz"
    if isinstance(dose_map, torch.Tensor):
        dose_map = dose_map.detach().cpu().numpy()
    dose_map = np.asarray(dose_map)
    if affine is None:
        affine = np.diag(list(voxel_size) + [1.0])
        center_offset = np.array(dose_map.shape) * np.array(voxel_size) / -2.0
        affine[:3, 3] = center_offset
    affine = np.asarray(affine, dtype=np.float64)
    metadata.update({
        "creation_date": "2025-02-08 09:50:56",
        "created_by": "devhliu",
        "voxel_size": voxel_size,
        "dimensions": dose_map.shape,
        "affine_matrix": affine.tolist(),
    })
    descrip = f"Created by {metadata['created_by']} at {metadata['creation_date']}"
    payload = _nifti_bytes(dose_map, voxel_size, affine, descrip, _json.dumps(metadata).encode("utf-8"))
    if filename.endswith(".gz"):
        with _gzip.open(filename, "wb") as f:
            f.write(payload)
    else:
        _Path(filename).write_bytes(payload)


def load_dose_map(filename):
    """Read a NIfTI-1 dose map (core/utils.py:105-152): returns (array, metadata)
    with voxel_size, dimensions, affine_matrix (sform when its code is set, else
    the qform, else the voxel-size diagonal), data_type, description, and the JSON
    of a code-44 extension merged in.  Any NIfTI-1 single file with a numeric data
    type loads; scl_slope / scl_inter are applied when set."""
    filename = str(filename)
    raw = _Path(filename).read_bytes()
    if raw[:2] == b"\x1f\x8b":
        raw = _gzip.decompress(raw)
    if len(raw) < _NIFTI_HDR + 4:
        raise ValueError(f"{filename}: too short for a NIfTI-1 header")
    end = "<" if _struct.unpack_from("<i", raw, 0)[0] == _NIFTI_HDR else ">"
    if _struct.unpack_from(end + "i", raw, 0)[0] != _NIFTI_HDR or raw[344:347] != b"n+1":
        raise ValueError(f"{filename}: not a single-file NIfTI-1 image")
    dim = _struct.unpack_from(end + "8h", raw, 40)
    datatype, bitpix = _struct.unpack_from(end + "hh", raw, 70)
    pixdim = _struct.unpack_from(end + "8f", raw, 76)
    vox_offset, slope, inter = _struct.unpack_from(end + "fff", raw, 108)
    descrip = raw[148:228].split(b"\x00", 1)[0].decode("utf-8", "replace")
    qform_code, sform_code = _struct.unpack_from(end + "hh", raw, 252)
    qb, qc, qd, qx, qy, qz = _struct.unpack_from(end + "6f", raw, 256)
    srow = np.array(_struct.unpack_from(end + "12f", raw, 280), dtype=np.float64).reshape(3, 4)
    if datatype not in _DT_NUMPY:
        raise ValueError(f"{filename}: unsupported NIfTI datatype {datatype}")
    nd = dim[0]
    shape = tuple(int(x) for x in dim[1:1 + nd])
    dt = np.dtype(_DT_NUMPY[datatype]).newbyteorder(end)
    count = int(np.prod(shape))
    data = np.frombuffer(raw, dtype=dt, count=count, offset=int(vox_offset)).reshape(shape, order="F")
    data = data.astype(dt.newbyteorder("="), copy=True)
    if slope not in (0.0,) and np.isfinite(slope) and (slope != 1.0 or (np.isfinite(inter) and inter != 0.0)):
        data = data * slope + (inter if np.isfinite(inter) else 0.0)
    if sform_code > 0:
        affine = np.vstack([srow, [0.0, 0.0, 0.0, 1.0]])
    elif qform_code > 0:
        qa = np.sqrt(max(0.0, 1.0 - (qb * qb + qc * qc + qd * qd)))
        rot = np.array([[qa * qa + qb * qb - qc * qc - qd * qd, 2 * (qb * qc - qa * qd), 2 * (qb * qd + qa * qc)],
                        [2 * (qb * qc + qa * qd), qa * qa + qc * qc - qb * qb - qd * qd, 2 * (qc * qd - qa * qb)],
                        [2 * (qb * qd - qa * qc), 2 * (qc * qd + qa * qb), qa * qa + qd * qd - qb * qb - qc * qc]])
        qfac = -1.0 if pixdim[0] < 0 else 1.0
        zooms = np.array([pixdim[1], pixdim[2], pixdim[3] * qfac])
        affine = np.eye(4)
        affine[:3, :3] = rot * zooms
        affine[:3, 3] = [qx, qy, qz]
    else:
        affine = np.diag([pixdim[1], pixdim[2], pixdim[3], 1.0])
    metadata = {
        "voxel_size": tuple(float(x) for x in pixdim[1:4]),
        "dimensions": data.shape,
        "affine_matrix": affine.tolist(),
        "data_type": str(np.dtype(_DT_NUMPY[datatype])),
        "description": descrip,
    }
    pos = _NIFTI_HDR + 4
    if raw[_NIFTI_HDR] != 0:
        while pos + 8 <= int(vox_offset):
            esize, ecode = _struct.unpack_from(end + "ii", raw, pos)
            if esize < 16 or pos + esize > int(vox_offset):
                break
            if ecode == 44:
                try:
                    metadata.update(_json.loads(raw[pos + 8:pos + esize].rstrip(b"\x00").decode("utf-8")))
                except ValueError:
                    pass
            pos += esize
    return data, metadata


# ---------------------------------------------------------------------------
# Resampling (core/utils.py:193-231, core/kernel_convolution.py:108-114)
# ---------------------------------------------------------------------------
def resampled_shape(shape, input_spacing, output_spacing) -> Tuple[int, ...]:
    """ceil(shape * input_spacing / output_spacing) per axis (the reference's output
    shape, core/utils.py:218-220), ignoring a rounding excess below 1e-9 voxel."""
    return tuple(int(np.ceil(n * float(a) / float(b) - 1e-9)) for n, a, b in zip(shape, input_spacing, output_spacing))


def resample_volume(volume, input_spacing, output_spacing, order: int = 3, conserve_total: bool = False,
                    output_shape=None, device=None):
    """Resample a 3-D volume from ``input_spacing`` to ``output_spacing`` (mm) on the GPU.

    Both grids share the volume's outer corner: input voxel i covers
    [i, i+1) * input_spacing, output voxel j is sampled at its centre
    (j + 0.5) * output_spacing.  ``order`` 3 is the interpolating cubic B-spline
    with mirror boundaries (scipy.ndimage.map_coordinates(order=3, mode='mirror')),
    1 trilinear.  ``conserve_total`` multiplies by the voxel-volume ratio, for
    extensive quantities such as activity per voxel (Bq): the total is then
    preserved to interpolation accuracy.  The output shape defaults to
    ``resampled_shape``.  Returns the caller's array kind.
    """
    from .. import _io
    if order not in (1, 3):
        raise ValueError("order must be 1 (trilinear) or 3 (cubic B-spline)")
    kind = _io.kind_of(volume)
    dev = _require_cuda(device if device is not None else (volume.device if kind == _io.CUDA_TENSOR else None))
    shape = tuple(volume.shape)
    if len(shape) != 3:
        raise ValueError("volume must be 3-D")
    inp = tuple(float(x) for x in input_spacing)
    outp = tuple(float(x) for x in output_spacing)
    if len(inp) != 3 or len(outp) != 3 or min(inp + outp) <= 0:
        raise ValueError("spacings must be three positive values")
    m = tuple(int(x) for x in (output_shape or resampled_shape(shape, inp, outp)))
    step = [b / a for a, b in zip(inp, outp)]
    origin = [0.5 * s - 0.5 for s in step]
    scale = float(np.prod(outp) / np.prod(inp)) if conserve_total else 1.0
    lib = N.load()
    with torch.cuda.device(dev):
        src = _io.to_device(volume, dev, "volume")
        sh = torch.cuda.current_stream(dev).cuda_stream
        if order == 3:
            coef = torch.empty_like(src)
            scratch = torch.empty_like(src)
            N.check(lib.pvd_bspline_prefilter(src.data_ptr(), coef.data_ptr(), scratch.data_ptr(), *shape, sh))
            del scratch
            src = coef
        out = torch.empty(m, dtype=torch.float32, device=dev)
        n_scr = shape[0] * shape[1] * m[2] + shape[0] * m[1] * m[2] + 8 * (m[0] + m[1] + m[2])
        scratch = torch.empty(max(n_scr, 1), dtype=torch.float32, device=dev)
        N.check(lib.pvd_resample_separable(src.data_ptr(), *shape, out.data_ptr(), *m, (C.c_double * 3)(*step),
                                           (C.c_double * 3)(*origin), order, scale, scratch.data_ptr(), n_scr, sh))
        return _io.from_device(out, kind)


def resample_dose_map(dose_map, input_spacing, output_spacing, order: int = 3):
    """The reference's resample_dose_map (core/utils.py:193-231): order-3 spline
    resampling to ``output_spacing``; returns (resampled, affine).  The input
    affine is the reference's diag(input_spacing) (voxel 0 at the origin); the
    returned affine places the output voxels on the same physical extent."""
    res = resample_volume(dose_map, input_spacing, output_spacing, order=order)
    aff = np.diag([float(x) for x in output_spacing] + [1.0])
    aff[:3, 3] = [0.5 * (float(b) - float(a)) for a, b in zip(input_spacing, output_spacing)]
    return res, aff
