"""The C-ABI library loads, exports every symbol include/gs3d.h declares, and
applies the reference's host-side validation and capacity policy (no GPU)."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT, pkg


@pytest.fixture(scope="module")
def lib():
    return pkg().load()


def declared_functions():
    with open(os.path.join(ROOT, "include", "gs3d.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w]+\**\s+\**(gs3d_\w+)\s*\(", text, re.M)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 14
    abi = __import__(pkg().__name__ + ".abi", fromlist=["SIGNATURES"])
    for name in names:
        assert hasattr(lib, name), name
        assert name in abi.SIGNATURES, f"{name} missing from the ctypes mirror"


def test_abi_version_and_defaults(lib):
    abi = __import__(pkg().__name__ + ".abi", fromlist=["PipelineDesc"])
    assert lib.gs3d_abi_version() == abi.GS3D_ABI_VERSION
    d = abi.PipelineDesc()
    lib.gs3d_pipeline_desc_defaults(C.byref(d))
    assert d.intersection_capacity == 262144
    assert d.raster_chunk_size == 8192
    assert abs(d.raster_transmittance_threshold - 1e-4) < 1e-9
    assert abs(d.depth_alpha_threshold - 0.95) < 1e-7
    assert abs(d.filter_variance - 0.3) < 1e-7
    assert d.subpixel_sample_culling == 1
    assert d.projection_precision == 0  # FP32: the reference's arithmetic


@pytest.mark.parametrize("field,value,status", [
    ("raster_chunk_size", 128, 2),            # rasterizationWGSL.test.ts:52-61
    ("raster_chunk_size", 1000, 2),
    ("raster_transmittance_threshold", 0.0, 2),  # GaussianPass.ts:245-253
    ("raster_transmittance_threshold", 1.0, 2),
    ("depth_alpha_threshold", 1.5, 2),           # GaussianPass.ts:231-238
    ("intersection_capacity", 0, 2),
    ("depth_sort_mode", 5, 1),
    ("projection_precision", 2, 1),
    ("abi_version", 99, 1),
])
def test_invalid_options_are_rejected_before_any_device_work(lib, field, value, status):
    abi = __import__(pkg().__name__ + ".abi", fromlist=["PipelineDesc"])
    d = abi.PipelineDesc()
    lib.gs3d_pipeline_desc_defaults(C.byref(d))
    setattr(d, field, value)
    data = abi.GaussianData()
    data.count, data.active_count, data.sh_degree = 4, 4, 3
    data.means = data.scales_opacity = data.rotations = data.sh_coefficients = 256
    out = C.c_void_p()
    assert lib.gs3d_pipeline_create(C.byref(d), C.byref(data), C.byref(out)) == status
    assert not out.value


def test_invalid_gaussian_data_is_rejected(lib):
    abi = __import__(pkg().__name__ + ".abi", fromlist=["PipelineDesc"])
    d = abi.PipelineDesc()
    lib.gs3d_pipeline_desc_defaults(C.byref(d))
    data = abi.GaussianData()
    out = C.c_void_p()
    data.count = 0
    assert lib.gs3d_pipeline_create(C.byref(d), C.byref(data), C.byref(out)) == abi.GS3D_ERROR_RANGE
    data.count, data.active_count, data.sh_degree = 4, 4, 4
    assert lib.gs3d_pipeline_create(C.byref(d), C.byref(data), C.byref(out)) == abi.GS3D_ERROR_RANGE
    data.sh_degree = 3
    assert lib.gs3d_pipeline_create(C.byref(d), C.byref(data), C.byref(out)) == abi.GS3D_ERROR_INVALID_ARGUMENT


def test_capacity_growth_policy(lib):
    # test/IntersectionCapacity.test.ts:26-38 (maximum 1000, growth 2, headroom 1.25)
    assert lib.gs3d_capacity_next(1000, 2.0, 1.25, 512, 900) == 1000
    assert lib.gs3d_capacity_next(1000, 2.0, 1.25, 1000, 1001) == 0
    # desired = max(ceil(300 * 1.25), 2 * 256) = 512, rounded to the 256 workgroup size
    assert lib.gs3d_capacity_next(10**6, 2.0, 1.25, 256, 300) == 512
    assert lib.gs3d_capacity_next(10**6, 2.0, 1.25, 256, 1000) == 1280


def test_null_arguments(lib):
    assert lib.gs3d_pipeline_create(None, None, None) == 1
    lib.gs3d_pipeline_destroy(None)
    assert lib.gs3d_pipeline_last_error(None) == b""
