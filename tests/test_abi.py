"""The C-ABI library: builds for sm_103a, loads, and exports every symbol that
include/*.h declares. Host-only entry points are exercised without a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(hl_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built_library):
    lib = C.CDLL(str(built_library))
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    from helio_gb300 import native as N

    assert set(N.EXPORTS) == declared_symbols()


def test_library_is_built_for_sm103a(built_library):
    from helio_gb300 import build as B

    assert "arch=compute_103a,code=sm_103a" in " ".join(B.ARCH)
    assert built_library.exists() and built_library.stat().st_size > 0


def test_abi_version_and_status_strings(built_library):
    from helio_gb300 import native as N

    l = N.load()
    assert l.hl_abi_version() == 1
    for s in (N.HL_OK, N.HL_ERR_INVALID_ARGUMENT, N.HL_ERR_LAYOUT, N.HL_ERR_SIZE, N.HL_ERR_CUDA, N.HL_ERR_TIMEOUT,
              N.HL_ERR_CAPACITY, N.HL_ERR_DEVICE_BOUNDS, N.HL_ERR_NOT_SUPPORTED):
        assert N.status_string(s) and N.status_string(s) != "unknown status"


def test_tile_count(built_library):
    from helio_gb300 import native as N

    l = N.load()
    assert l.hl_tile_count(1920, 1080) == 120 * 68
    assert l.hl_tile_count(1, 1) == 1
    assert l.hl_tile_count(0, 10) == 0
    assert l.hl_tile_count(0xFFFFFFFF, 0xFFFFFFFF) == 0  # "tile grid overflow"


def test_slice_table_matches_oracle(built_library, oracle_lib):
    from helio_gb300 import layouts as L
    from helio_gb300 import native as N

    for grid in [(16, 9, 24), (32, 18, 48), (1, 1, 1), (8, 8, 128)]:
        p = N.froxel_params(*grid, 1920, 1080, 100.0)
        got = np.array(N.slice_table(p), np.float32)
        want = oracle_lib.froxel_slice_table(L.froxel_params(*grid, 1920, 1080, 100.0))
        np.testing.assert_array_equal(got, want)
        assert got[0] == 0 and got[-1] == 100.0 and np.all(np.diff(got) > 0)


def test_slice_table_rejects_bad_params(built_library):
    from helio_gb300 import native as N

    for bad in [N.froxel_params(0, 9, 24, 1920, 1080, 100.0), N.froxel_params(16, 9, 129, 1920, 1080, 100.0),
                N.froxel_params(16, 9, 24, 1920, 1080, 100.0, slice_near=0.0)]:
        with pytest.raises(N.HelioError):
            N.slice_table(bad)


def test_create_fails_loudly_without_gpu(built_library):
    import torch

    from helio_gb300 import native as N

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(N.HelioError) as e:
        N.Context(0)
    assert e.value.status == N.HL_ERR_CUDA


def test_entry_points_reject_null_context(built_library):
    from helio_gb300 import native as N

    l = N.load()
    assert l.hl_bin_tiles_ref(None, None, None, 0, 16, 16, None, None, None) == N.HL_ERR_INVALID_ARGUMENT
    assert l.hl_sync_status(None, None) == N.HL_ERR_INVALID_ARGUMENT
    assert l.hl_destroy(None) == N.HL_OK
