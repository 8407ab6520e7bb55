"""The C-ABI library builds, loads and exports every declared symbol (no GPU)."""

import ctypes
import os
import re

import pytest

from horton_part_gb300 import _lib
from horton_part_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "hpgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|const char\*)\s+(hp_\w+)\(", text, re.M)))


@pytest.fixture(scope="module")
def library():
    build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_declarations_found():
    syms = declared_symbols()
    assert "hp_job_create" in syms and "hp_step" in syms and len(syms) >= 12


def test_every_declared_symbol_is_exported(library):
    for name in declared_symbols():
        assert hasattr(library, name), name


def test_binding_covers_header():
    assert set(declared_symbols()) <= set(_lib.EXPORTED)


def test_abi_version(library):
    assert _lib.lib().hp_abi_version() == 4


def test_struct_sizes_match_header():
    # natural alignment on LP64: hp_job_desc is 4*4 + 2*8 + 9*8 + 6*8 + 4*4 bytes,
    # then nrad (4 + 4 padding) and five atom-grid pointers
    assert ctypes.sizeof(_lib.JobDesc) == 16 + 16 + 72 + 48 + 16 + 8 + 40
    assert ctypes.sizeof(_lib.JobResults) == 8 * 8


def test_job_info_fields_match_header():
    # member names of hp_job_info, in declaration order, against the binding
    text = open(os.path.join(ROOT, "include", "hpgpu.h")).read()
    body = re.search(r"typedef struct \{([^{}]*)\} hp_job_info;", text).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = re.findall(r"^\s*\w+\s+(\w+);", body, re.M)
    assert names == [f[0] for f in _lib.JobInfo._fields_]
    assert "f64_factors" in names


def test_invalid_arguments_fail_before_device_work(library):
    L = _lib.lib()
    assert L.hp_job_create(None, None, None) == _lib.HP_ERR_INVALID
    assert L.hp_step(None, None, 0, None) == _lib.HP_ERR_INVALID
    assert L.hp_job_info_get(None, None) == _lib.HP_ERR_INVALID
    assert b"null" in L.hp_last_error()
