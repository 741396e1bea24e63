"""The C-ABI library without a GPU: it loads, exports every symbol that
include/tdbem.h declares, and refuses to run (no CPU fallback)."""
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "tdbem.h")).read()
    return sorted(set(re.findall(r"\b(tdbem_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import build as b  # td-bem_gb300/build.py
    b.build()
    from tdbem import lib as L
    return L.load()


def test_library_exports_every_declared_symbol(lib):
    from tdbem import lib as L
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(L.SIGNATURES)


def test_version_string(lib):
    assert b"sm_103a" in lib.tdbem_version()


def test_null_arguments_are_rejected(lib):
    assert lib.tdbem_ctx_create(None, None, 1.0, 6, 0, None) == -1
    assert lib.tdbem_max_step(None, None) == -1
    assert b"null" in lib.tdbem_last_error()
