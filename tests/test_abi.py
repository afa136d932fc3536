"""The C-ABI libraries load and export every symbol their headers declare
(no device compute here)."""

import ctypes
import os
import re

import pytest

from taurus_vap_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tv[as]p?_[a-z0-9_]+)\s*\(", text)))


def test_gpu_library_exports_header():
    path = _build.build_gpu()
    L = ctypes.CDLL(path)
    names = declared("tvap.h")
    assert "tvap_calculate_fields" in names and "tvap_project" in names
    for name in names:
        assert hasattr(L, name), name


def test_setup_library_exports_header():
    L = ctypes.CDLL(_build.build_setup())
    for name in declared("tvap_setup.h"):
        assert hasattr(L, name), name


def test_every_status_code_has_a_message():
    """The binding names every status code the header declares."""
    from taurus_vap_gb300 import native

    text = open(os.path.join(ROOT, "include", "tvap.h")).read()
    codes = {int(v) for v in re.findall(r"\bTVAP_ERR_[A-Z0-9_]+\s*=\s*(\d+)", text)}
    assert codes and 19 in codes
    assert codes <= set(native.ERRORS), sorted(codes - set(native.ERRORS))
    err = native.TvapError(19, "tvap_project", "detail")
    assert err.code == 19 and "bounded wait" in str(err) and "detail" in str(err)
