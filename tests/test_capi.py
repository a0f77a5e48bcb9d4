"""The C ABI library builds, loads and exports everything the header
declares; host-side error paths that need no GPU (no compute calls)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "nssdmrg.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = set(re.findall(r"\b(nss_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    from nssdmrg_gb300 import build
    return build.build()


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ["nss_create", "nss_destroy", "nss_last_error", "nss_sb_upload", "nss_hv", "nss_eigh",
                 "nss_rdm", "nss_sb_setup", "nss_dmrg_create"]:
        assert must in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(str(libpath))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(libpath):
    import nssdmrg_gb300 as nss
    L = nss.lib()
    for n in declared_functions():
        assert getattr(L, n).argtypes is not None or getattr(L, n).restype is not None, n


def test_create_without_gpu_fails_cleanly(libpath):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import nssdmrg_gb300 as nss
    L = nss.lib()
    ctx = L.nss_create(0, 0)
    assert not ctx
    assert b"no CUDA device" in L.nss_last_error(None)


def test_null_context_is_an_error_not_a_crash(libpath):
    import nssdmrg_gb300 as nss
    L = nss.lib()
    assert L.nss_hv(None, 4, None, None) == nss.NSS_ERR_INVALID
    assert L.nss_sb_dim(None) == 0


def test_server_and_batch_without_gpu_fail_cleanly(libpath):
    """Without a device the server is not created (no threads are left
    running), and the batch and server entry points refuse NULL handles."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import nssdmrg_gb300 as nss
    L = nss.lib()
    assert not L.nss_server_create(0, 1 << 30)
    assert not L.nss_batch_create(None)
    assert L.nss_batch_step(None, 1, None, None, None, None) == nss.NSS_ERR_INVALID
    assert L.nss_batch_inflight(None) == 0
    assert L.nss_server_submit(None, None, None) == nss.NSS_ERR_INVALID
    assert L.nss_server_solves(None) == 0
    L.nss_server_destroy(None)
    L.nss_batch_destroy(None)
