"""CPU tests of the C ABI surface: the library loads, exports every symbol
include/mnad.h declares, the Python binding covers them all, and argument
checks that need no GPU return the documented status codes."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import mnad
from mnad import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mnad.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"MNAD_API\s+[\w\s\*]+?\b(mnad_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def L():
    from mnad import build
    build.build()
    return _lib.lib()


def test_header_declares_the_drop_in_entry_points():
    names = declared()
    for n in ("mnad_fwd_pde_exact", "mnad_born_adj", "mnad_context_create", "mnad_last_error",
              "mnad_wavefield_export", "mnad_wavefield_import", "mnad_run_jobs", "mnad_plan_run"):
        assert n in names


def test_library_exports_every_declared_symbol(L):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\bT\s+(mnad_\w+)", out.stdout))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    # nothing else leaks out of the library
    assert exported == set(declared())


def test_binding_covers_every_declared_symbol(L):
    assert set(_lib.SIGNATURES) == set(declared())
    for name in declared():
        assert getattr(L, name) is not None


def test_abi_version(L):
    assert L.mnad_abi_version() == 1


def test_null_arguments_are_rejected_without_a_gpu(L):
    d = np.zeros(4)
    p = d.ctypes.data_as(C.POINTER(C.c_double))
    rc = L.mnad_fwd_pde_exact(None, 10.0, 1.0, p, 1, 10.0, 1.0, p, p, 2, 2, 1e-3, 1, p, 0, 1, 0, p, None, None)
    assert rc == _lib.E_ARG
    assert b"context" in L.mnad_last_error()
    assert L.mnad_born_adj(None, 1.0, 1.0, 1, 1e-3, p, 2, 2, p, p, 1, p, 0, 1, p) == _lib.E_ARG
    assert L.mnad_context_create(0, 0, None) == _lib.E_ARG
    assert L.mnad_plan_run(None) == _lib.E_ARG
    assert L.mnad_run_jobs(None, None, 0) == _lib.E_ARG


def test_errors_map_to_matlab_style_identifiers(L):
    with pytest.raises(mnad.MnadError) as ei:
        _lib.check(L.mnad_plan_run(None))
    assert ei.value.identifier == "mnad:arg"
    assert ei.value.code == _lib.E_ARG


def test_options_struct_matches_header():
    src = open(HEADER).read()
    body = re.search(r"typedef struct mnad_options \{(.*?)\} mnad_options;", src, re.S).group(1)
    fields = re.findall(r"int\s+(\w+);", body)
    assert fields == [f for f, _ in _lib.Options._fields_]
    body = re.search(r"typedef struct mnad_job \{(.*?)\} mnad_job;", src, re.S).group(1)
    fields = re.findall(r"(?:int|double|const double\*|double\*)\s+(\w+)(?:,\s*(\w+))?(?:,\s*(\w+))?(?:,\s*(\w+))?;",
                        body)
    flat = [x for tup in fields for x in tup if x]
    assert flat == [f for f, _ in _lib.Job._fields_]


def test_enum_constants_match_header():
    """Every MNAD_* enumerator of the header has the same value in the
    Python binding (status codes, codecs, pairings, kernels, job kinds and
    states)."""
    src = open(HEADER).read()
    header = {}
    for body in re.findall(r"enum\s*\{(.*?)\}", src, re.S):
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        for name, val in re.findall(r"MNAD_(\w+)\s*=\s*(\d+)", body):
            header[name] = int(val)
    assert len(header) >= 24
    for name, val in header.items():
        assert getattr(_lib, name) == val, name


def test_server_structs_match_header():
    src = open(HEADER).read()
    body = re.search(r"typedef struct mnad_server_options \{(.*?)\} mnad_server_options;", src, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"(?:size_t|int)\s+(\w+);", body)
    assert fields == [f for f, _ in _lib.ServerOptions._fields_]
    body = re.search(r"typedef struct mnad_server_stats \{(.*?)\} mnad_server_stats;", src, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in re.findall(r"(?:int64_t|double|size_t)\s+([\w\s,]+);", body):
        fields += [f.strip() for f in decl.split(",")]
    assert fields == [f for f, _ in _lib.ServerStats._fields_]
