"""The C-ABI library: it loads without a GPU and exports every function
include/swm_gpu.h declares, and the ctypes binding covers all of them.
No compute call is made (there may be no GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'swm_gpu.h')


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', ' ', text, flags=re.S)
    names = re.findall(r'^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;', text, flags=re.M)
    return sorted(set(n for n in names if n not in ('if', 'while')))


@pytest.fixture(scope='module')
def library():
    from swm_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from swm_gb300 import build
        build.build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ('swm_gpu_create', 'swm_gpu_step', 'swm_gpu_advance', 'swm_gpu_run', 'trc_gpu_add',
              'elsolv_sor_gpu_solve', 'swm_gpu_integrals_noalloc'):
        assert n in names, n
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(library):
    missing = [n for n in declared_functions() if not hasattr(library, n)]
    assert not missing, missing


def test_ctypes_binding_covers_the_header():
    from swm_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_create_without_gpu_fails_loudly(library):
    """With no visible device, swm_gpu_create returns an error code and a
    message instead of falling back to the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is visible')
    from swm_gb300 import _lib
    L = _lib.lib()
    cfg = _lib.Config(nx=8, ny=8, dt=1.0)
    ctx = ctypes.c_void_p()
    rc = L.swm_gpu_create(ctypes.byref(cfg), ctypes.byref(ctx))
    assert rc != 0
    assert b'device' in L.swm_gpu_last_error().lower()
