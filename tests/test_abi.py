"""The C-ABI library loads and exports every symbol include/nerfgb.h declares;
argument validation answers without touching a GPU (no CPU device needed)."""
import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "nerfgb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nerfgb_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib(ng):
    return ng._lib.lib()


def test_every_declared_symbol_is_exported_and_bound(lib, ng):
    syms = declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(ng._lib.SIGNATURES), set(syms) - set(ng._lib.SIGNATURES)


def test_version_and_status_strings(lib, ng):
    assert lib.nerfgb_abi_version() == 2
    assert ng._lib.status_name(0) == "NERFGB_OK"
    assert ng._lib.status_name(-4) == "NERFGB_E_TIMEOUT"
    assert ng._lib.status_name(-99) == "NERFGB_E_UNKNOWN"


def test_param_and_pack_sizes(lib, ng):
    assert lib.nerfgb_mlp_param_count() == ng.weights.PARAM_COUNT == 595844
    # fp32 pack: padded K (64,256x4,320,256x3,288) weights + bias/head table
    assert lib.nerfgb_mlp_packed_bytes(0) == (593920 + 2432 + 256 + 4 + 384 + 4) * 4
    assert lib.nerfgb_mlp_packed_bytes(1) >= 593920 * 2
    assert lib.nerfgb_mlp_packed_bytes(7) == -1


def test_workspace_bytes(lib):
    b = lib.nerfgb_render_workspace_bytes(4096, 64, 128)
    assert b >= 4096 * (64 * 11 + 192 * 8) * 4
    assert lib.nerfgb_render_workspace_bytes(-1, 64, 128) == -1


def test_argument_validation_without_device(lib, ng):
    E = ng._lib
    # zero rays: nothing to launch
    assert lib.nerfgb_coarse_sample(None, None, None, None, None, 0, 64, 1, 1,
                                    None, None, None, None, None, None) == E.OK
    assert lib.nerfgb_coarse_sample(None, None, None, None, None, -1, 64, 1, 1,
                                    None, None, None, None, None, None) == E.E_INVALID_ARG
    assert lib.nerfgb_coarse_sample(None, None, None, None, None, 4, 2000, 1, 1,
                                    None, None, None, None, None, None) == E.E_UNSUPPORTED
    assert lib.nerfgb_coarse_sample(None, None, None, None, None, 4, 64, 1, 1,
                                    None, None, None, None, None, None) == E.E_INVALID_ARG
    assert lib.nerfgb_fine_sample(None, None, None, None, 65, None, None, None, 4, 64, 1024,
                                  None, None, None, None, None, None) == E.E_UNSUPPORTED
    assert lib.nerfgb_fine_sample(None, None, None, None, 10, None, None, None, 4, 64, 128,
                                  None, None, None, None, None, None) == E.E_INVALID_ARG
    assert lib.nerfgb_composite(None, None, None, 4, 64, 0, 5, None, None, None, None,
                                None) == E.E_UNSUPPORTED
    assert lib.nerfgb_composite(None, None, None, 4, 64, 0, 1, None, None, None, None,
                                None) == E.E_INVALID_ARG
    assert lib.nerfgb_mlp_forward(None, 3, None, None, 10, 1, None, None, None,
                                  None) == E.E_UNSUPPORTED
    assert lib.nerfgb_mlp_forward(None, 0, None, None, 10, 0, None, None, None,
                                  None) == E.E_INVALID_ARG
    assert lib.nerfgb_mlp_forward(None, 1, None, None, 0, 1, None, None, None, None) == E.OK
    # misaligned pack buffer
    assert lib.nerfgb_mlp_pack(ctypes.c_void_p(256), 0, ctypes.c_void_p(0x1001), None) == E.E_INVALID_ARG
    assert lib.nerfgb_positional_encode(None, 5, 20, None, None) == E.E_UNSUPPORTED
    assert lib.nerfgb_uniform(1, 0, -1, None, None) == E.E_INVALID_ARG
    assert lib.nerfgb_render_rays(None, None, 0, None, None, None, None, None, None, 0, 8, 64, 128,
                                  1, 1, 0, 1, None, None, None, None, None, None, None, None,
                                  None) == E.E_INVALID_ARG


def test_error_mapping(ng):
    with pytest.raises(ng.NerfgbError) as ei:
        ng._lib.call("nerfgb_uniform", 1, 0, -1, None, None)
    assert ei.value.code == "NERFGB_E_INVALID_ARG"
