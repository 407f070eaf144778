"""The C ABI library builds, loads and exports what include/nlmgpu.h declares.

No GPU is needed: the symbols are resolved, no compute entry point is called
(except nlm_device_count / argument validation, which touch no kernel).
"""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from nlmech_gb300 import abi, build, gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def declared(header):
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nlm_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return gpu.load()


def test_exports_every_declared_symbol(lib):
    names = []
    for h in HEADERS:
        names += declared(h)
    assert len(names) > 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(lib):
    assert lib.nlm_abi_version() == 1


def test_struct_layout_matches_header():
    """ctypes mirrors of the description structs have the C sizes/offsets."""
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "nlmgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(nlm_bc_set), sizeof(nlm_crack),
         sizeof(nlm_material), sizeof(nlm_fd_desc));
  printf("%zu %zu %zu %zu %zu\n", offsetof(nlm_fd_desc, material), offsetof(nlm_fd_desc, ubc),
         offsetof(nlm_fd_desc, dt), offsetof(nlm_fd_desc, u0), offsetof(nlm_material, es_sc));
  printf("%zu %zu %zu\n", sizeof(nlm_esqs_params), offsetof(nlm_esqs_params, lin_tol),
         offsetof(nlm_esqs_params, dt));
  printf("%zu %zu %zu\n", sizeof(nlm_qs_params), offsetof(nlm_qs_params, wait_limit_s),
         offsetof(nlm_qs_params, lin_tol_gamma));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    sizes = [C.sizeof(abi.BCSet), C.sizeof(abi.Crack), C.sizeof(abi.Material), C.sizeof(abi.FDDesc)]
    offs = [abi.FDDesc.material.offset, abi.FDDesc.ubc.offset, abi.FDDesc.dt.offset,
            abi.FDDesc.u0.offset, abi.Material.es_sc.offset]
    esqs = [C.sizeof(abi.ESQSParams), abi.ESQSParams.lin_tol.offset, abi.ESQSParams.dt.offset]
    qs = [C.sizeof(abi.QSParams), abi.QSParams.wait_limit_s.offset,
          abi.QSParams.lin_tol_gamma.offset]
    assert [int(v) for v in out] == sizes + offs + esqs + qs


def test_invalid_arguments_are_status_codes(lib):
    """Bad descriptions return NLM_ERR_* with a message; nothing exits."""
    h = C.c_void_p()
    assert lib.nlm_fd_create(None, C.byref(h)) == abi.NLM_ERR_INVALID
    assert lib.nlm_last_error()
    d = abi.FDDesc()
    d.dim = 5
    assert lib.nlm_fd_create(C.byref(d), C.byref(h)) == abi.NLM_ERR_UNSUPPORTED
    d.dim = 2
    d.n_nodes = 0
    assert lib.nlm_fd_create(C.byref(d), C.byref(h)) == abi.NLM_ERR_INVALID
    rp = (C.c_int64 * 2)()
    assert lib.nlm_neighbor_search(C.c_int(2), C.c_int64(-1), None, C.c_double(1.0), rp, None) \
        == abi.NLM_ERR_INVALID


def test_nonfinite_input_rejected_before_gpu_use(lib):
    import numpy as np
    from nlmech_gb300 import configs
    p = configs.rnp_plate(8, 1e-3, 3, 0.0, 0.1, 2e-8, 1)
    p.x = p.x.copy()
    p.x[3, 0] = np.nan
    d, keep = p.desc()
    h = C.c_void_p()
    assert lib.nlm_fd_create(C.byref(d), C.byref(h)) == abi.NLM_ERR_NONFINITE


def test_device_count_without_gpu_is_not_an_error(lib):
    c = C.c_int(-1)
    assert lib.nlm_device_count(C.byref(c)) == 0
    assert c.value >= 0
