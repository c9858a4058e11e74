"""NIfTI-1 dose maps (the reference's save_dose_map / load_dose_map,
core/utils.py:53-152, which go through nibabel — absent here, so the format is
checked against the NIfTI-1 header layout itself with an independent parse)."""
import gzip
import json
import struct

import numpy as np
import pytest


def parse(raw):
    """Independent reading of the fields the writer sets (NIfTI-1 layout)."""
    f = {}
    f["sizeof_hdr"] = struct.unpack_from("<i", raw, 0)[0]
    f["dim"] = struct.unpack_from("<8h", raw, 40)
    f["datatype"], f["bitpix"] = struct.unpack_from("<hh", raw, 70)
    f["pixdim"] = struct.unpack_from("<8f", raw, 76)
    f["vox_offset"] = struct.unpack_from("<f", raw, 108)[0]
    f["descrip"] = raw[148:228].split(b"\0")[0].decode()
    f["qform_code"], f["sform_code"] = struct.unpack_from("<hh", raw, 252)
    f["srow"] = np.array(struct.unpack_from("<12f", raw, 280)).reshape(3, 4)
    f["magic"] = raw[344:348]
    f["ext_flag"] = raw[348]
    f["esize"], f["ecode"] = struct.unpack_from("<ii", raw, 352)
    f["ext"] = raw[360:352 + f["esize"]]
    return f


@pytest.mark.parametrize("gz", [True, False])
def test_layout_and_round_trip(tmp_path, gz):
    from pyvoxeldosimetry_gb300.core.utils import load_dose_map, save_dose_map
    rng = np.random.default_rng(1)
    dose = rng.random((7, 9, 11)).astype(np.float64) * 50.0
    md = {"radionuclide": "Lu177", "method": "kernel_convolution"}
    name = tmp_path / ("d.nii.gz" if gz else "d.nii")
    save_dose_map(name, dose, (1.5, 2.0, 2.5), md)
    raw = name.read_bytes()
    if gz:
        assert raw[:2] == b"\x1f\x8b"
        raw = gzip.decompress(raw)
    f = parse(raw)
    assert f["sizeof_hdr"] == 348 and f["magic"] == b"n+1\0"
    assert f["dim"][:4] == (3, 7, 9, 11) and f["datatype"] == 16 and f["bitpix"] == 32
    assert f["pixdim"][1:4] == (1.5, 2.0, 2.5) and f["pixdim"][0] == 1.0
    assert f["sform_code"] == 2
    aff = np.diag([1.5, 2.0, 2.5, 1.0])
    aff[:3, 3] = -np.array([7, 9, 11]) * np.array([1.5, 2.0, 2.5]) / 2
    np.testing.assert_allclose(f["srow"], aff[:3], rtol=0, atol=1e-6)
    assert f["ext_flag"] == 1 and f["ecode"] == 44 and f["esize"] % 16 == 0
    assert f["vox_offset"] == 352 + f["esize"] and f["vox_offset"] % 16 == 0
    meta = json.loads(f["ext"].rstrip(b"\0"))
    assert meta["radionuclide"] == "Lu177" and meta["created_by"] == "devhliu"
    assert f["descrip"] == "Created by devhliu at 2025-02-08 09:50:56"
    body = np.frombuffer(raw, "<f4", offset=int(f["vox_offset"])).reshape((7, 9, 11), order="F")
    np.testing.assert_array_equal(body, dose.astype(np.float32))
    # the reference updates the caller's metadata dict in place
    assert md["voxel_size"] == (1.5, 2.0, 2.5) and md["dimensions"] == (7, 9, 11)
    d2, m2 = load_dose_map(name)
    np.testing.assert_array_equal(d2, dose.astype(np.float32))
    assert m2["data_type"] == "float32" and m2["radionuclide"] == "Lu177"
    assert m2["voxel_size"] == [1.5, 2.0, 2.5]        # from the JSON extension, as in the reference
    np.testing.assert_allclose(np.array(m2["affine_matrix"]), aff, atol=1e-6)


def test_name_without_extension_gets_nii_gz(tmp_path):
    from pyvoxeldosimetry_gb300.core.utils import save_dose_map
    save_dose_map(tmp_path / "dose", np.zeros((2, 3, 4), np.float32), (1.0, 1.0, 1.0), {})
    assert (tmp_path / "dose.nii.gz").exists()


def test_qform_encodes_a_rotated_reflected_affine(tmp_path):
    from pyvoxeldosimetry_gb300.core.utils import load_dose_map, save_dose_map
    rng = np.random.default_rng(7)
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    if np.linalg.det(q) > 0:
        q[:, 0] = -q[:, 0]                       # a reflection: qfac = -1
    aff = np.eye(4)
    aff[:3, :3] = q * np.array([1.2, 0.8, 2.5])
    aff[:3, 3] = [10.0, -20.0, 5.5]
    p = tmp_path / "rot.nii"
    save_dose_map(p, np.ones((3, 4, 5), np.float32), (1.2, 0.8, 2.5), {}, affine=aff)
    raw = bytearray(p.read_bytes())
    assert struct.unpack_from("<8f", raw, 76)[0] == -1.0
    # drop the JSON extension (its copy of the affine would override the header's) and keep
    # only the qform, so the loaded affine is rebuilt from quaternion, voxel sizes and qfac
    esize = struct.unpack_from("<i", raw, 352)[0]
    raw = raw[:348] + b"\0\0\0\0" + raw[352 + esize:]
    struct.pack_into("<f", raw, 108, 352.0)
    struct.pack_into("<hh", raw, 252, 1, 0)
    p.write_bytes(bytes(raw))
    _, m = load_dose_map(p)
    np.testing.assert_allclose(np.array(m["affine_matrix"]), aff, atol=2e-6)


def test_reads_big_endian_int16_with_scaling(tmp_path):
    from pyvoxeldosimetry_gb300.core.utils import load_dose_map
    h = bytearray(348)
    struct.pack_into(">i", h, 0, 348)
    struct.pack_into(">8h", h, 40, 3, 2, 3, 4, 1, 1, 1, 1)
    struct.pack_into(">hh", h, 70, 4, 16)
    struct.pack_into(">8f", h, 76, 1, 2, 2, 2, 0, 0, 0, 0)
    struct.pack_into(">fff", h, 108, 352.0, 0.5, 10.0)
    h[344:348] = b"n+1\0"
    vals = np.arange(24, dtype=">i2").reshape((2, 3, 4), order="F")
    (tmp_path / "be.nii").write_bytes(bytes(h) + b"\0\0\0\0" + vals.tobytes(order="F"))
    d, m = load_dose_map(tmp_path / "be.nii")
    np.testing.assert_array_equal(d, vals.astype(np.float64) * 0.5 + 10.0)
    assert m["voxel_size"] == (2.0, 2.0, 2.0) and m["data_type"] == "int16"
