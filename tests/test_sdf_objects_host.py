"""SDF objects and the SDF volume cache without a GPU: the C object layout, the
reference's volume fill (oracle/_ref) on known values, and the scene file
carrying SDF fields and volumes."""
import ctypes as C

import numpy as np
import pytest

from aperturerendererv3_gb300 import _lib
from aperturerendererv3_gb300.scene import AdditionalObjectInfo, Material, SceneObject, sdf
from oracle import ref_runner as rr


def test_object_layout_carries_the_sdf_fields():
    assert C.sizeof(_lib.ArObject) == 104
    assert _lib.ArObject.sdf_type.offset == 80 and _lib.ArObject.sdf_volume.offset == 100
    assert sdf.CreateTorus(2.0) == AdditionalObjectInfo(_lib.SDF_OBJECT_TORUS, (0.75, 0.25, 0.0, 0.0))
    assert sdf.CreateSDFVolume(3).volume == 3 and sdf.CreateSDFVolume(3).sdf_type == _lib.SDF_OBJECT_VOLUME


@pytest.fixture(scope="module")
def ref_available():
    if not rr.available():
        pytest.skip("reference oracle not built in this checkout")


def test_reference_torus_volume_known_values(ref_available):
    # 33^3 grid over [-0.5, 0.5]^3: voxel 16 is the centre; (R, r) = (0.375, 0.125)
    v = rr.sdf_volume(_lib.SDF_FN_TORUS, (0.375, 0.125, 0.0, 0.0), (33, 33, 33))
    assert v.shape == (33, 33, 33)
    assert abs(v[16, 16, 16] - (0.375 - 0.125)) < 1e-6           # centre: distance R - r
    assert abs(v[16, 16, 28] - (-0.125)) < 1e-6                  # on the ring (x = 0.375): -r
    assert np.isclose(v[16, 16, 32], 0.125 - 0.125 + 0.0, atol=1e-6)  # x = 0.5: 0.125 from the ring, r = 0.125


def test_reference_diamond_volume_is_a_closed_shape(ref_available):
    v = rr.sdf_volume(_lib.SDF_FN_DIAMOND, sdf.CreateDiamond(), (32, 32, 32))
    assert v[16, 16, 16] < 0.0                                   # inside at the centre
    assert (v[[0, -1], :, :] > 0.0).all() and (v[:, :, [0, -1]] > 0.0).all()  # outside at the faces


def test_scene_file_with_sdf_objects_and_volumes():
    obj = SceneObject((0.0, 0.0, 0.0), (0.3, 0.2, 0.3), Material(), (10.0, 0.0, 0.0), _lib.OBJECT_SDF,
                      sdf.CreateSDFVolume(1))
    data = np.arange(24, dtype=np.float32).reshape(2, 3, 4)
    b = rr.scene_bytes([obj], volumes=[(_lib.SDF_FN_TORUS, (0.3, 0.1, 0.0, 0.0), (8, 8, 8)), (None, data, None)])
    assert b[:4] == b"ARS2"
    rec = np.frombuffer(b[8: 8 + rr.OBJ_DTYPE.itemsize], rr.OBJ_DTYPE)[0]
    assert rec["type"] == 2 and rec["sdf_type"] == 1 and rec["sdf_volume"] == 1
    at = 8 + rr.OBJ_DTYPE.itemsize
    assert np.frombuffer(b[at: at + 4], np.int32)[0] == 2
    tail = b[at + 4 + 2 * rr.VOL_DTYPE.itemsize:]
    assert np.array_equal(np.frombuffer(tail, np.float32), data.reshape(-1))
