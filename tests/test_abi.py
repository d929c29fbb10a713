"""CPU-only checks of the C ABI: the library builds, loads without a GPU, exports every
entry point include/bvpgpu.h declares, and validates arguments before touching CUDA."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "bvpgpu.h")) as f:
        txt = f.read()
    return sorted(set(re.findall(r"\b(bvp_[a-z_]+)\s*\(", txt)))


def test_header_and_binding_agree(pkg):
    assert sorted(pkg.EXPORTS) == _declared()


def test_library_exports_every_declared_symbol(pkg):
    lib = C.CDLL(pkg.build_library())
    for name in _declared():
        assert hasattr(lib, name), name


def test_default_options_are_the_reference_defaults(pkg):
    lib = pkg.load_library()
    o = pkg._lib.Options()
    lib.bvp_default_options(C.byref(o))
    assert o.abstol == 1e-6 and o.adaptive == 1           # mirk.jl:50
    assert o.defect_threshold == 0.1                       # calc_errors.jl:54-60
    assert o.max_subintervals == 3000                      # algorithms.jl:60
    assert o.order == 4 and o.transfer_inplace == 1 and o.bc_jac_exact == 0


@pytest.mark.parametrize("field,value", [("M", 0), ("M", 9), ("n_bc_pts", 0), ("n_bc_pts", 17)])
def test_create_rejects_bad_descriptions_without_cuda(pkg, problems, field, value):
    lib = pkg.load_library()
    p = problems.PENDULUM
    d = pkg._lib.ProblemDesc()
    d.M, d.n_params, d.twopoint, d.n_bc_pts = p.M, p.n_params, 0, 2
    setattr(d, field, value)
    h = C.c_void_p()
    st = lib.bvp_create(C.byref(d), p.source.encode(), None, C.byref(h))
    assert st == 1 and not h.value


def test_create_rejects_bad_two_point_split(pkg, problems):
    lib = pkg.load_library()
    p = problems.SINGULAR_PERTURBATION
    d = pkg._lib.ProblemDesc()
    d.M, d.n_params, d.twopoint, d.La, d.Lb = 2, 1, 1, 1, 2
    h = C.c_void_p()
    assert lib.bvp_create(C.byref(d), p.source.encode(), None, C.byref(h)) == 1


def test_device_code_compiles_for_sm103a(pkg):
    # build_library() ran nvcc -cubin for sm_103a on the kernel sources; its ptxas report
    # must exist and show no local-memory spills growing without bound
    path = pkg.build_library()
    rep = os.path.join(os.path.dirname(path), "ptxas_pendulum_o4.txt")
    txt = open(rep).read()
    assert "bvp_solve_fused" in txt and "sm_103a" in txt


def test_destroy_releases_every_buffer_of_the_handle():
    # every device and pinned host buffer the handle owns is released by bvp_destroy
    import re
    src = open(os.path.join(ROOT, "boundaryvaluediffeq.jl_gb300", "csrc", "bvpgpu_host.cpp")).read()
    start = src.index("struct bvp_handle_s {")
    decl = src[start:src.index("};", start)]
    body = src[src.index("void bvp_destroy(bvp_handle* h) {"):]
    body = body[:body.index("delete h;")]
    freed = set(re.findall(r"&h->(\w+)", body))
    for kind in ("DevBuf", "HostBuf"):
        for m in re.finditer(kind + r" ([^;]+);", decl):
            for name in (x.strip() for x in m.group(1).replace("\n", " ").split(",")):
                assert name in freed, name
