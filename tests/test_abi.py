"""The C ABI library builds for sm_103a, loads without a GPU, and exports every
function include/nemo_gpu.h declares (no compute call is made here)."""
import ctypes as C

import pytest

from nemo_gpu import _ffi, build as nbuild
from oracle import build as obuild


@pytest.fixture(scope="module")
def lib_path():
    return nbuild.build()


def test_library_exports_every_header_symbol(lib_path):
    lib = _ffi.load(lib_path)
    syms = _ffi.header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_field_ids_match_header():
    assert _ffi.F["TSB"] == 0
    assert _ffi.F["COUNT"] == len(_ffi.F) - 1
    assert set(_ffi.FP64_FIELDS) <= set(_ffi.F)


def test_struct_layout():
    # nemo_dom_desc: 4 ints then 17 pointers; nemo_namelist: mixed doubles/ints
    assert C.sizeof(_ffi.DomDesc) == 16 + 17 * 8
    assert _ffi.Namelist.rn_aht_0.offset % 8 == 0


def test_oracle_builds_and_exports():
    lib = C.CDLL(obuild.build())
    for s in ("ora_create", "ora_tra_adv_fct", "ora_tra_ldf_iso", "ora_tra_zdf_imp", "ora_dyn_spg_ts",
              "ora_lbc_lnk", "ora_glob_sum", "ora_stp_hotpath"):
        assert hasattr(lib, s)
