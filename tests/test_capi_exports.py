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
