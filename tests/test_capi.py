"""CPU checks of the C ABI: the library builds, loads and exports every declared symbol."""
import ctypes as C
import os
import re

import pytest

from maestroex_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(madv_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    build.build_library()
    L = C.CDLL(capi.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(L, n), n
    assert sorted(names) == sorted(capi.EXPORTED)


def test_version_string():
    build.build_library()
    assert b"sm_103a" in capi.lib().madv_version()


def test_params_struct_matches_oracle_layout():
    import pyoracle  # noqa: F401  (oracle header uses the same field order)
    from maestroex_gb300.params import MadvParams
    hdr = open(os.path.join(ROOT, "include", "maestro_adv.h")).read()
    body = hdr[hdr.index("typedef struct {\n    int nspec;"):hdr.index("} madv_params;")]
    fields = re.findall(r"^\s*(?:int|double)\s+(\w+)", body, flags=re.M)
    assert fields == [f[0] for f in MadvParams._fields_]
    ohdr = open(os.path.join(ROOT, "oracle", "maestro_oracle.h")).read()
    obody = ohdr[ohdr.index("typedef struct {\n    int nspec;"):ohdr.index("} mo_params;")]
    assert re.findall(r"^\s*(?:int|double)\s+(\w+)", obody, flags=re.M) == fields
