"""CPU tests of the C ABI: the library loads without a GPU, exports every symbol the headers
declare, and its host-side size helpers match the reference's known answers and the oracle."""
import json
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = json.loads((ROOT / "tests/golden/known_answers.json").read_text())


def declared_functions(header: Path) -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = re.findall(r"\b(vren_[a-z0-9_]+)\s*\(", text)
    # drop macro-like and typedef names; keep those that look like declarations
    return sorted(set(n for n in names if not n.endswith("_t")))


def test_library_exports_every_declared_symbol(native):
    for header in sorted((ROOT / "include").glob("vren_gb300*.h")):
        for name in declared_functions(header):
            assert hasattr(native, name), f"{name} declared in {header.name} but not exported"


def test_scene_library_exports(native):
    import ctypes

    from vren_gb300 import _build

    scene = ctypes.CDLL(str(_build.SCENE_LIB))
    for name in declared_functions(ROOT / "include/vren_scene.h"):
        assert hasattr(scene, name), name


def test_bvh_size_helpers_known_answers(native):
    kn = GOLDEN["bvh_size_helpers"]
    for n, v in kn["padded_leaf_count"].items():
        assert native.vren_calc_bvh_padded_leaf_count(int(n)) == v
    for n, v in kn["buffer_length"].items():
        assert native.vren_calc_bvh_buffer_length(int(n)) == v
    for n, v in kn["root_index"].items():
        assert native.vren_calc_bvh_root_index(int(n)) == v
    for n, v in kn["level_count"].items():
        assert native.vren_calc_bvh_level_count(int(n)) == v


def test_size_helpers_match_oracle_formulas(native):
    import oracle

    rng = np.random.default_rng(7)
    ns = [0, 1, 2, 31, 32, 33, 1023, 1024, 1025, 32767, 32768, 32769, 2**20, 2**20 + 1, 2**25, 2**30]
    ns += [int(x) for x in rng.integers(0, 2**30, 300)]
    ol = oracle.lib()
    for n in ns:
        assert native.vren_calc_bvh_padded_leaf_count(n) == ol.oracle_calc_bvh_padded_leaf_count(n), n
        assert native.vren_calc_bvh_buffer_length(n) == ol.oracle_calc_bvh_buffer_length(n), n
        assert native.vren_calc_bvh_root_index(n) == ol.oracle_calc_bvh_root_index(n), n
        assert native.vren_calc_bvh_level_count(n) == ol.oracle_calc_bvh_level_count(n), n
        assert native.vren_round_to_next_power_of_2(n) == ol.oracle_round_to_next_power_of_2(n), n
        for d in (1, 3, 32, 1024):
            assert native.vren_divide_and_ceil(n, d) == ol.oracle_divide_and_ceil(n, d), (n, d)
        for b in (2, 32):
            if n > 0:
                assert native.vren_round_to_next_power_of(n, b) == ol.oracle_round_to_next_power_of(n, b), (n, b)


def test_bucket_sort_scratch_covers_the_one_scatter_layout(native):
    """For up to 10 key bits the scratch holds the one-scatter form's layout: 2,064 header words
    (scan ticket and counters, bucket totals, bucket starts), a 1,024-word count row per
    4,096-element tile and a 1,024-word look-back row per block of 256 tile rows; and it covers the
    radix-pass form too, which either key width may select."""
    for n in [0, 1, 4096, 4097, 1 << 20, (1 << 24) + 5, (1 << 26) + 12345, (1 << 30) - 1]:
        rows = max(1, -(-n // 4096))
        blocks = -(-rows // 256)
        one_scatter = (2064 + (rows + blocks) * 1024) * 4
        for kb in (1, 7, 10):
            assert native.vren_bucket_sort_scratch_bytes(n, kb) >= one_scatter, (n, kb)
        assert native.vren_bucket_sort_scratch_bytes(n, 16) > 0
    assert native.vren_bucket_sort_scratch_bytes(100, 0) == 0
    assert native.vren_bucket_sort_scratch_bytes(100, 17) == 0


def test_status_strings(native):
    assert native.vren_status_string(0) == b"ok"
    assert native.vren_status_string(2) == b"capacity exceeded"


def test_argument_errors_need_no_gpu(native):
    # validation happens before any CUDA call
    assert native.vren_radix_sort_u32(None, None, 1000, None, None) == 1   # not a power of two
    assert native.vren_radix_sort_u32(None, None, 512, None, None) == 1    # below 1024
    assert native.vren_build_bvh(None, None, 33) == 1
    assert native.vren_scan_downsweep_u32(None, None, 3, 1, 1) == 1
    assert native.vren_bucket_sort_u32x2(None, None, 10, None, 17, None) == 1


@pytest.mark.parametrize("W,H", [(640, 360), (1280, 720), (1920, 1080), (2560, 1440), (100, 37)])
@pytest.mark.parametrize("slicing", ["ref", "fixed32"])
def test_slice_tables_match_oracle(native, W, H, slicing):
    import oracle
    import vren_gb300.clustered_shading as cs

    view = cs.view_from_camera(cs.scene_camera(W, H), slicing)
    f = cs.frame_build(view, W, H)
    near, far = oracle.cs_slice_table(view, (H + 31) // 32)
    assert np.array_equal(np.array(f.slice_near, np.float32), near)
    assert np.array_equal(np.array(f.slice_far, np.float32), far)
    assert f.tiles_x == (W + 31) // 32 and f.tiles_y == (H + 31) // 32
    assert f.max_slice == (31 if slicing == "fixed32" else 1023)
    head = near[: f.max_slice + 1]
    assert np.all(head[1:] >= head[:-1])  # non-decreasing (+inf once a^k overflows)


def test_camera_matrices(native):
    import vren_gb300.clustered_shading as cs

    cam = cs.scene_camera(1920, 1080, near=0.1, far=1000.0)
    v = cs.view_from_camera(cam)
    view = np.array(v.view, np.float64).reshape(4, 4).T  # row-major
    assert np.allclose(view, np.eye(4))
    inv_proj = np.array(v.inv_proj, np.float64).reshape(4, 4).T
    t = np.tan(np.float32(np.deg2rad(45.0)) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0] = 1 / (t * 1920 / 1080)
    proj[1, 1] = 1 / t
    proj[2, 2] = 1000 / (1000 - 0.1)
    proj[2, 3] = -(1000 * 0.1) / (1000 - 0.1)
    proj[3, 2] = 1
    assert np.allclose(inv_proj @ proj, np.eye(4), atol=1e-5)
    # a moved camera: view * inv_view = I
    cam2 = cs.scene_camera(640, 360, position=(1, 2, 3), yaw=0.4, pitch=0.1)
    v2 = cs.view_from_camera(cam2)
    a = np.array(v2.view, np.float64).reshape(4, 4).T
    b = np.array(v2.inv_view, np.float64).reshape(4, 4).T
    assert np.allclose(a @ b, np.eye(4), atol=1e-5)
