"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
entry point that include/*.h declares (no compute calls)."""
import ctypes
import glob
import os
import re

import pytest

from nimblesm_gb300 import build as B
from nimblesm_gb300 import engine as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(nsm_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    B.build()
    return E.library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_binding_signatures_cover_the_header(lib):
    assert declared_functions() == set(E.SIGNATURES)


def test_abi_version_without_gpu(lib):
    assert lib.nsm_abi_version() == 1


def test_library_is_sm_103a():
    # the fatbin carries sm_103a code; cuobjdump is not used (no disassembly):
    # the build flags are checked instead
    assert "arch=compute_103a,code=sm_103a" in " ".join(B.ARCH)
