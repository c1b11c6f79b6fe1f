"""CPU tests of the C-ABI boundary: libsi_cuda loads, exports every function include/si_cuda.h
declares, and its host helpers reproduce the reference's JavaScript host arithmetic bit for bit
(mpm.js:38-46, 148-199, 683-714). No GPU: nothing here launches a kernel."""
import ctypes
import os
import re

import numpy as np
import pytest

import host_ref
from shaderintel_gb300 import _lib as L
from shaderintel_gb300 import mpm as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "si_cuda.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\s*\*)\s*\*?\s*(si_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_function():
    lib = L.lib()
    names = header_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(L.SIGNATURES), "ctypes signatures out of step with the header"
    assert b"sm_103a" in lib.si_version()


def test_library_is_in_tree_cuda_build():
    from shaderintel_gb300 import build
    assert os.path.dirname(build.LIB).startswith(os.path.join(ROOT, "shaderintel_gb300"))
    assert os.path.exists(build.LIB)


@pytest.mark.parametrize("name", list(M.MATERIALS))
@pytest.mark.parametrize("ppc", [1, 2, 3])
def test_material_rows_match_reference_host_math(name, ppc):
    d = dict(M.MATERIALS[name])
    got = M.material_row(d, ppc)
    want = host_ref.material_row(d, ppc)
    assert got.view(np.uint32).tolist() == want.view(np.uint32).tolist()


def test_material_validation_errors():
    with pytest.raises(L.SIError) as e:
        M.material_row({"kind": 0, "density": 1000})
    assert e.value.code == "invalid-argument" and "density" in str(e.value)
    with pytest.raises(L.SIError):
        M.material_row({"kind": 7})
    row = M.material_row({"kind": 1, "poisson": 0.5, "stiffness": 0.5})   # clamped to 0.49, finite
    assert np.isfinite(row).all()


@pytest.mark.parametrize("shape", [
    {"box": [[0.1, 0.2, 0.3], [0.35, 0.4, 0.45]]},
    {"sphere": [[0.5, 0.5, 0.5], 0.13]},
    {"cylinder": [[0.5, 0.4, 0.5], 0.1, 0.07]},
])
@pytest.mark.parametrize("seed", [1, 77, 0xFFFFFFFF])
def test_sample_shape_matches_reference(shape, seed):
    got = M.sample_shape(shape, 1 / 64, 0.6, seed)
    want = host_ref.sample_shape(shape, 1 / 64, 0.6, seed)
    assert got.shape == want.shape and len(got) > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_sample_shape_sdf_path_matches_box():
    sdf = {"sdf": lambda p: -1.0, "bounds": [[0.1, 0.1, 0.1], [0.2, 0.25, 0.2]]}
    a = M.sample_shape(sdf, 1 / 48, 0.6, 9)
    b = host_ref.sample_shape({"box": [[0.1, 0.1, 0.1], [0.2, 0.25, 0.2]]}, 1 / 48, 0.6, 9)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_geometry_matches_constructor():
    for grid, size in [(32, 1), (48, 1), (64, [1, 0.5, 2]), (128, 1), (96, 1)]:
        g = host_ref.geometry(grid, size)
        assert min(g["dims"]) >= 8


def test_no_device_fails_loudly():
    """Without a GPU the product refuses to run instead of falling back to the CPU."""
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a device is present")
    h = ctypes.c_void_p()
    rc = L.lib().si_world_create(ctypes.byref(h))
    assert rc == L.SI_EDEVICE
    with pytest.raises(L.SIError) as e:
        M.MPM(grid=16, maxParticles=1024)
    assert e.value.code == "no-device"
