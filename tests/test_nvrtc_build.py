"""The kernels compile through NVRTC for sm_103a exactly as bvp_create compiles them (same
source assembly and options), for every MIRK order and MIRK6I, both Jacobian precisions, standard and
two-point problems, the larger-state family, a problem with a singular term, the build
with the global-error controllers and the block-mode module. NVRTC runs on
the CPU, so this catches JIT-only compile errors without a GPU."""
import pytest


def _nvrtc_available(pkg):
    return pkg._lib._nvrtc() is not None


CASES = [
    ("pendulum", 2, 32), ("pendulum", 3, 32), ("pendulum", 5, 64), ("pendulum", 6, 32),
    ("multipoint", 4, 32), ("affine_twopoint", 3, 64), ("torus", 4, 32),
    ("lane_emden", 6, 64), ("nonlinear32", 6, 32), ("nonlinear32", 4, 64), ("nonlinear32", 3, 32), ("mathieu", 4, 32),
    ("pendulum", 6, 32, 1), ("singular_perturbation", 6, 64, 1), ("nonlinear32", 6, 32, 1),
    # the build with the global-error controllers (BVP_GLOBAL_CTL), and the MIRK(p+2) module of HO
    ("torus", 4, 64, 0, 1), ("pendulum", 6, 32, 0, 1),
    # the block-mode module for long meshes (BVP_BLOCK_MODE), interior BCs and two-point
    ("singular_perturbation", 6, 32, 0, 0, 0, 1), ("pendulum", 4, 64, 0, 0, 0, 1),
]


def test_kernels_compile_with_nvrtc(pkg, problems):
    if not _nvrtc_available(pkg):
        pytest.skip("libnvrtc not found")
    from concurrent.futures import ThreadPoolExecutor   # NVRTC releases the GIL
    with ThreadPoolExecutor(max_workers=8) as ex:
        futs = {case: ex.submit(pkg._lib.nvrtc_check, problems.ALL[case[0]], *case[1:]) for case in CASES}
        for case, f in futs.items():
            f.result()   # raises with the NVRTC log for the failing case


def test_nvrtc_check_reports_errors(pkg, problems):
    if not _nvrtc_available(pkg):
        pytest.skip("libnvrtc not found")
    from dataclasses import replace
    bad = replace(problems.PENDULUM, source=problems.PENDULUM.source + "\nBVP_SING { su[0] = undefined_name; }\n")
    with pytest.raises(RuntimeError, match="NVRTC build check failed"):
        pkg._lib.nvrtc_check(bad, 4, 32)
