"""The C ABI library: it loads, exports every entry point include/gbp.h declares, and refuses to run without
an sm_103 GPU (there is no CPU fallback).  No compute calls are made here."""
import ctypes
import os
import re
import subprocess

import pytest

from scip_gb300 import gbp
from scip_gb300.build import LIBGBP, build_libgbp

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gbp.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(gbp_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    build_libgbp()
    return gbp.load_library()


def test_header_and_binding_agree():
    assert declared() == sorted(gbp.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", LIBGBP], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(gbp_\w+)", out))
    missing = [s for s in declared() if s not in exported]
    assert not missing, f"missing exports: {missing}"
    for s in declared():
        assert getattr(lib, s) is not None


def test_error_strings(lib):
    assert lib.gbp_version() >= 1
    assert lib.gbp_error_string(gbp.GBP_ERR_NODEVICE).decode() == "no suitable CUDA device"
    assert lib.gbp_error_string(gbp.GBP_ERR_TOO_LARGE).decode() == "problem too large for the no-alloc scratch"


def test_default_params_are_scips(lib):
    p = gbp.default_params()
    assert (p.infinity, p.epsilon, p.sumepsilon, p.feastol, p.hugeval, p.boundstreps, p.recompfac) == \
           (1e20, 1e-9, 1e-6, 1e-6, 1e15, 0.05, 1e6)
    assert p.maxeasyactivitydelta == 1e6


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_no_device_fails_loudly(lib):
    with pytest.raises(gbp.GbpError) as e:
        gbp.Propagator(0)
    assert e.value.code == gbp.GBP_ERR_NODEVICE


def test_noalloc_argument_checks_need_no_device(lib):
    res = gbp.GbpResult()
    # negative sizes and null pointers are rejected before anything touches a device
    rc = lib.gbp_propagate_nodes_noalloc(-1, 10, *([None] * 11), 1, *([None] * 11), 0, None, None, ctypes.byref(res))
    assert rc == gbp.GBP_ERR_INVALID
    rc = lib.gbp_propagate_nodes_noalloc(10, 10, *([None] * 11), 1, *([None] * 11), 0, None, None, ctypes.byref(res))
    assert rc == gbp.GBP_ERR_INVALID


def test_server_argument_checks_need_no_device(lib):
    """The serving loop's calls reject bad arguments before anything touches a device, and a server cannot be
    created without one."""
    import numpy as np

    h = ctypes.c_void_p()
    par = gbp.default_params()
    # no workers, a negative cap, missing root bounds
    assert lib.gbp_server_create(ctypes.byref(h), 0, 0, 0, 16, 0, ctypes.byref(par), 1, 1, *([None] * 8)) == \
        gbp.GBP_ERR_INVALID
    assert lib.gbp_server_create(ctypes.byref(h), 0, 1, 0, 16, -1, ctypes.byref(par), 1, 1, *([None] * 8)) == \
        gbp.GBP_ERR_INVALID
    assert lib.gbp_server_create(ctypes.byref(h), 0, 1, 0, 16, 0, ctypes.byref(par), 1, 1, *([None] * 8)) == \
        gbp.GBP_ERR_INVALID
    assert lib.gbp_server_submit(None, 0, None, None, None, None) == gbp.GBP_ERR_INVALID
    assert lib.gbp_server_submit_instance(None, 0, 0, *([None] * 8), None) == gbp.GBP_ERR_INVALID
    assert lib.gbp_server_destroy(None) == gbp.GBP_ERR_INVALID
    assert lib.gbp_error_string(gbp.GBP_ERR_BUSY).decode() == "reply not ready"
    if not _has_gpu():
        from scip_gb300 import instances

        inst = instances.root_mip(0, m=50, n=100)
        with pytest.raises(gbp.GbpError) as e:
            gbp.Server(inst, inst.lb, inst.ub, workers=1)
        assert e.value.code == gbp.GBP_ERR_NODEVICE
        assert np.isfinite(inst.lb).all()
