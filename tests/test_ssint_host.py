"""The surface-interaction boundary's argument checks, on the CPU.

ffea_gpu_ssint_create validates its descriptor on the host before any
device work: each malformed input below is refused with FFEA_ERROR and a
message naming the fault (surfaced by ffea_gb300.surface as FfeaGpuError),
and the Python mirror refuses malformed parameter tables itself.
"""
import numpy as np
import pytest

from ffea_gb300 import _lib as L
from ffea_gb300 import surface as S

# two triangles of one blob over four nodes, one interaction type
FACES = np.array([[0, 1, 2], [1, 2, 3]], np.int32)
GOOD = dict(num_nodes=4, faces=FACES, face_blob=np.zeros(2, np.int32), face_type=np.zeros(2, np.int32),
            emin=np.ones((1, 1)), rmin=np.ones((1, 1)), num_blobs=1, cell_size=1.0, grid=(4, 4, 4))


@pytest.fixture(scope="module", autouse=True)
def built():
    from ffea_gb300 import build as B
    B.build()


def make(**over):
    kw = dict(GOOD)
    kw.update(over)
    return S.SurfaceSolver(**kw)


@pytest.mark.parametrize("over,match", [
    (dict(faces=np.array([[0, 1, 2], [1, 2, 4]], np.int32)), "node 4 out of range"),
    (dict(faces=np.array([[0, 1, 2], [1, -1, 3]], np.int32)), "node -1 out of range"),
    (dict(face_type=np.array([0, 1], np.int32)), "interaction type 1 >= num_types"),
    (dict(face_blob=np.array([0, 1], np.int32)), "blob 1 out of range"),
    (dict(cell_size=0.0), "cell_size must be positive"),
    (dict(grid=(4, 0, 4)), "grid dimensions must be positive"),
    (dict(grid=(1024, 1024, 1024)), "cells exceed the maximum"),
    (dict(num_blobs=0), "no types or blobs"),
    (dict(ssint_type=7), "unknown ssint_type 7"),
    (dict(ssint_type=S.SSINT_STERIC), "need face_apex"),
    (dict(ssint_type=S.SSINT_STERIC, face_apex=np.array([3, 0], np.int32), steric_dr=0.0), "steric_dr must be positive"),
    (dict(ssint_type=S.SSINT_STERIC, face_apex=np.array([3, 9], np.int32)), "node 9 out of range"),
    (dict(ssint_type=S.SSINT_GENSOFT, face_apex=np.array([3, 0], np.int32)), "gensoft needs k0"),
])
def test_create_refuses_malformed_descriptors(over, match):
    with pytest.raises(L.FfeaGpuError, match=match):
        make(**over)


def test_inactive_faces_are_not_checked_against_the_type_table():
    """A face of type -1 is not in the interaction pool (FFEA leaves it out),
    so its type is never looked up: only the active faces' fields are
    validated, and the first active face's error is the one reported."""
    with pytest.raises(L.FfeaGpuError, match="face 1: node 7 out of range"):
        make(face_type=np.array([-1, 0], np.int32), faces=np.array([[0, 1, 2], [1, 2, 7]], np.int32))


@pytest.mark.parametrize("over,match", [
    (dict(emin=np.ones((1, 2))), "square"),
    (dict(rmin=np.ones((2, 2))), "square"),
    (dict(ssint_type=S.SSINT_GENSOFT, face_apex=np.array([3, 0], np.int32), k0=np.ones((2, 2))), "k0 must be"),
])
def test_python_mirror_refuses_malformed_tables(over, match):
    with pytest.raises(ValueError, match=match):
        make(**over)
