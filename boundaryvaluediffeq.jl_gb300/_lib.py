"""Build and ctypes binding of libbvpgpu.so (the C ABI of include/bvpgpu.h).

The library is built in-tree into ``_build/``: the device headers are embedded as raw
strings (NVRTC compiles them at ``bvp_create`` together with the problem source), the host
runtime is compiled by nvcc and linked against the static CUDA runtime and NVRTC, and the
device code is additionally compiled once by nvcc for sm_103a as a build check (its
``-Xptxas -v`` report goes to ``_build/ptxas_<problem>.txt``).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
import threading

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD = os.path.join(PKG_DIR, "_build")
INCLUDE = os.path.join(os.path.dirname(PKG_DIR), "include")
LIB_PATH = os.path.join(BUILD, "libbvpgpu.so")
EMBED = ("bvp_prelude.cuh", "bvp_kernels.cuh", "bvp_large.cuh", "bvp_shared.h", "bvp_tableau.cuh", "bvp_firk.cuh")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

_lock = threading.Lock()
_lib = None


def _write_embedded() -> str:
    h = hashlib.sha256()
    parts = []
    for fn in EMBED:
        with open(os.path.join(CSRC, fn)) as f:
            txt = f.read()
        if ")BVPRAW\"" in txt:
            raise RuntimeError(f"raw-string delimiter inside {fn}")
        h.update(txt.encode())
        parts.append((fn, txt))
    out = ["// generated by _lib.py: device sources embedded for NVRTC", f"static const int kEmbedCount = {len(parts)};"]
    out.append("static const char* kEmbedNames[] = {" + ", ".join(f'"{fn}"' for fn, _ in parts) + "};")
    out.append("static const char* kEmbedSources[] = {")
    for fn, txt in parts:
        out.append(f'R"BVPRAW({txt})BVPRAW",')
    out.append("};")
    out.append(f'static const char* kEmbedHash = "{h.hexdigest()[:32]}";')
    path = os.path.join(BUILD, "bvp_embedded.inc")
    body = "\n".join(out) + "\n"
    if not os.path.exists(path) or open(path).read() != body:
        with open(path, "w") as f:
            f.write(body)
    return h.hexdigest()


def _sources_digest() -> str:
    h = hashlib.sha256()
    for fn in sorted(os.listdir(CSRC)):
        with open(os.path.join(CSRC, fn), "rb") as f:
            h.update(fn.encode())
            h.update(f.read())
    with open(os.path.join(INCLUDE, "bvpgpu.h"), "rb") as f:
        h.update(f.read())
    with open(__file__, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def _run(cmd, log=None):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if log:
        with open(log, "w") as f:
            f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _nvrtc():
    for name in ("libnvrtc.so", "libnvrtc.so.13", os.path.join(os.path.dirname(NVCC), "..", "lib64", "libnvrtc.so")):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


def nvrtc_check(problem, order: int, jac_bits: int = 32, mirk6i: int = 0, global_ctl: int = 0,
                firk_stages: int = 0, block_mode: int = 0) -> None:
    """Compile the problem's kernels with NVRTC exactly as bvp_create does (same source
    assembly and options, no GPU needed; global_ctl: the build with the error controllers other
    than DefectControl; firk_stages: the FIRK path's build for that many stages, with
    placeholder coefficients; block_mode: the block-mode module for long meshes); raises with the
    NVRTC log on failure."""
    lib = _nvrtc()
    if lib is None:
        return
    large = problem.M > 8
    nbc = 2 if problem.twopoint else len(problem.bc_t)
    prefix = ""
    if firk_stages:
        s = firk_stages
        row = "{" + ", ".join(["0.5"] * s) + "}"
        prefix = ("#define BVP_FIRK 1\nnamespace bvp {\n"
                  f"constexpr int FS = {s}, FORDER = {2 * s - 1};\nconstexpr double FTAU = 0.0;\n"
                  f"constexpr double FC[{s}] = {row};\nconstexpr double FB[{s}] = {row};\n"
                  f"constexpr double FA[{s}][{s}] = {{{', '.join([row] * s)}}};\n"
                  f"constexpr double FQ[{s}][{s}] = {{{', '.join([row] * s)}}};\n}}\n")
    if block_mode:
        prefix += "#define BVP_BLOCK_MODE 1\n"
    src = ("#include \"bvp_prelude.cuh\"\n" + prefix + "#line 1 \"problem_source\"\n" + problem.source +
           ("\n#include \"bvp_large.cuh\"\n" if large else "\n#include \"bvp_kernels.cuh\"\n"))
    opts = ["--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "--fmad=true", f"-DBVP_M={problem.M}",
            f"-DBVP_ORDER={order}", f"-DBVP_TWOPOINT={int(problem.twopoint)}", f"-DBVP_NBC={nbc}",
            f"-DBVP_LA={problem.La if problem.twopoint else 0}",
            "-DBVP_JT=" + ("double" if jac_bits == 64 else "float"), f"-DBVP_MIRK6I={int(bool(mirk6i))}",
            f"-DBVP_SINGULAR={int('BVP_SING' in problem.source)}"] + (["-DBVP_GLOBAL_CTL=1"] if global_ctl else [])
    names = [fn.encode() for fn in EMBED]
    bodies = [open(os.path.join(CSRC, fn), "rb").read() for fn in EMBED]
    prog = C.c_void_p()
    arr = lambda xs: (C.c_char_p * len(xs))(*xs)
    if lib.nvrtcCreateProgram(C.byref(prog), src.encode(), b"bvp_problem.cu", len(EMBED), arr(bodies), arr(names)):
        raise RuntimeError("nvrtcCreateProgram failed")
    try:
        rc = lib.nvrtcCompileProgram(prog, len(opts), arr([o.encode() for o in opts]))
        n = C.c_size_t()
        lib.nvrtcGetProgramLogSize(prog, C.byref(n))
        log = C.create_string_buffer(n.value)
        lib.nvrtcGetProgramLog(prog, log)
        if rc != 0:
            raise RuntimeError(f"NVRTC build check failed ({problem.name}, MIRK{order}, JT {jac_bits}):\n"
                               + log.value.decode(errors="replace"))
    finally:
        lib.nvrtcDestroyProgram(C.byref(prog))


def device_check_source(problem) -> str:
    """A translation unit with the problem inlined, for the nvcc sm_103a build check."""
    kernels = "bvp_large.cuh" if problem.M > 8 else "bvp_kernels.cuh"
    return ("#include \"bvp_prelude.cuh\"\n" + problem.source + f"\n#include \"{kernels}\"\n")


def build_library(verbose: bool = False, force: bool = False, check_problems=None) -> str:
    """Compile libbvpgpu.so (host runtime) and nvcc-check the device code for sm_103a."""
    from . import problems as P
    os.makedirs(BUILD, exist_ok=True)
    with _lock:
        digest = _sources_digest()
        stamp = os.path.join(BUILD, "libbvpgpu.stamp")
        if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp) and open(stamp).read() == digest:
            return LIB_PATH
        _write_embedded()
        jobs = []
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        host_cmd = [NVCC, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", ARCH, "-lineinfo",
                    "-I", INCLUDE, "-I", CSRC, "-I", BUILD, os.path.join(CSRC, "bvpgpu_host.cpp"),
                    os.path.join(CSRC, "bvp_mlp.cu"), "-o", tmp, "-lnvrtc", "-ldl"]
        jobs.append(subprocess.Popen(host_cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
        checks = check_problems if check_problems is not None else [
            (P.PENDULUM, 4, 0), (P.SINGULAR_PERTURBATION, 6, 0), (P.NONLINEAR32, 4, 0), (P.LANE_EMDEN, 4, 0)]
        check_cmds = []
        for prob, order, nbc_dummy in checks:
            src = os.path.join(BUILD, f"check_{prob.name}_o{order}.cu")
            with open(src, "w") as f:
                f.write(device_check_source(prob))
            nbc = 2 if prob.twopoint else len(prob.bc_t)
            cmd = [NVCC, "-cubin", ARCH, "-std=c++17", "-lineinfo", "-O3", "-Xptxas", "-v",
                   f"-DBVP_M={prob.M}", f"-DBVP_ORDER={order}", f"-DBVP_TWOPOINT={int(prob.twopoint)}",
                   f"-DBVP_NBC={nbc}", f"-DBVP_LA={prob.La}", "-DBVP_JT=float",
                   f"-DBVP_SINGULAR={int('BVP_SING' in prob.source)}", "-I", CSRC, src,
                   "-o", os.path.join(BUILD, f"check_{prob.name}_o{order}.cubin")]
            check_cmds.append((cmd, os.path.join(BUILD, f"ptxas_{prob.name}_o{order}.txt")))
            jobs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
        # the same kernels through NVRTC (what bvp_create runs), in both Jacobian precisions
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=4) as ex:
            futs = [ex.submit(nvrtc_check, prob, order, bits) for prob, order, _ in checks for bits in (32, 64)]
            for f in futs:
                f.result()
        outs = [j.communicate()[0] for j in jobs]
        if jobs[0].returncode != 0:
            raise RuntimeError("host library build failed:\n" + " ".join(host_cmd) + "\n" + outs[0])
        for (cmd, log), j, o in zip(check_cmds, jobs[1:], outs[1:]):
            with open(log, "w") as f:
                f.write(" ".join(cmd) + "\n" + o)
            if j.returncode != 0:
                raise RuntimeError("sm_103a device build check failed:\n" + " ".join(cmd) + "\n" + o)
            if verbose:
                print(o.strip().splitlines()[-1] if o.strip() else "")
        os.replace(tmp, LIB_PATH)
        with open(stamp, "w") as f:
            f.write(digest)
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


# ---- ctypes mirror of include/bvpgpu.h ----------------------------------------------------

class ProblemDesc(C.Structure):
    _fields_ = [("M", C.c_int32), ("n_params", C.c_int32), ("twopoint", C.c_int32),
                ("n_bc_pts", C.c_int32), ("La", C.c_int32), ("Lb", C.c_int32),
                ("bc_t", C.c_double * 16)]


class Options(C.Structure):
    _fields_ = [("order", C.c_int32), ("adaptive", C.c_int32), ("max_subintervals", C.c_int32),
                ("max_newton", C.c_int32), ("max_rounds", C.c_int32), ("transfer_inplace", C.c_int32),
                ("bc_jac_exact", C.c_int32), ("linesearch_fallback", C.c_int32),
                ("stall_steps", C.c_int32), ("jac_precision", C.c_int32), ("want_stages", C.c_int32),
                ("fp32_phase", C.c_int32), ("abstol", C.c_double), ("defect_threshold", C.c_double),
                ("divergence_factor", C.c_double), ("mirk6i", C.c_int32),
                ("controller", C.c_int32), ("global_method", C.c_int32),
                ("hybrid_de", C.c_double), ("hybrid_ge", C.c_double),
                ("firk", C.c_int32), ("firk_stages", C.c_int32), ("block_min", C.c_int32)]


# bvp_controller and bvp_global_method
CONTROLLERS = {"defect": 0, "global": 1, "sequential": 2, "hybrid": 3}
GLOBAL_METHODS = {"HO": 0, "RE": 1}
# bvp_options.firk
FIRK_FAMILIES = {"RadauIIa": 1, "LobattoIIIa": 2, "LobattoIIIb": 3, "LobattoIIIc": 4}


class Results(C.Structure):
    _fields_ = [("retcode", C.POINTER(C.c_int32)), ("n_nodes", C.POINTER(C.c_int32)),
                ("newton_iters", C.POINTER(C.c_int32)), ("rounds", C.POINTER(C.c_int32)),
                ("defect", C.POINTER(C.c_double)), ("resid", C.POINTER(C.c_double)),
                ("global_err", C.POINTER(C.c_double))]


EXPORTS = ("bvp_default_options", "bvp_create", "bvp_solve_batch", "bvp_solve_batch_device",
           "bvp_solve_batch_device_grid",
           "bvp_fetch_results", "bvp_get_solution", "bvp_get_packed", "bvp_eval_stage",
           "bvp_dense_output", "bvp_mlp_create", "bvp_mlp_num_params", "bvp_mlp_set_params",
           "bvp_mlp_get_params", "bvp_mlp_set_normalization", "bvp_mlp_forward", "bvp_mlp_loss_grad",
           "bvp_mlp_train", "bvp_mlp_forward_device", "bvp_mlp_forward_noalloc", "bvp_resample_guess_device",
           "bvp_mlp_destroy",
           "bvp_solve_batch_warm", "bvp_solve_batch_device_warm", "bvp_get_fused_tuning", "bvp_get_block_mode",
           "bvp_last_timing", "bvp_get_tuning", "bvp_get_work_order", "bvp_stream", "bvp_last_error",
           "bvp_destroy")


def load_library(path: str | None = None):
    """Load libbvpgpu.so (building it if needed) and declare the C signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or build_library()
    lib = C.CDLL(path)
    vp, i32, f64p, i32p = C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int32)
    lib.bvp_default_options.argtypes = [C.POINTER(Options)]
    lib.bvp_default_options.restype = None
    lib.bvp_create.argtypes = [C.POINTER(ProblemDesc), C.c_char_p, C.POINTER(Options), C.POINTER(vp)]
    lib.bvp_create.restype = C.c_int
    lib.bvp_solve_batch.argtypes = [vp, i32, f64p, i32p, f64p, i32, f64p, C.POINTER(Results)]
    lib.bvp_solve_batch.restype = C.c_int
    lib.bvp_solve_batch_device.argtypes = [vp, i32, vp, vp, vp, i32, vp, vp, i32]
    lib.bvp_solve_batch_device.restype = C.c_int
    lib.bvp_solve_batch_device_grid.argtypes = [vp, i32, vp, vp, vp, vp, i32, i32]
    lib.bvp_solve_batch_device_grid.restype = C.c_int
    lib.bvp_fetch_results.argtypes = [vp, C.POINTER(Results)]
    lib.bvp_fetch_results.restype = C.c_int
    lib.bvp_get_solution.argtypes = [vp, i32, f64p, f64p, i32, i32p]
    lib.bvp_get_solution.restype = C.c_int
    lib.bvp_get_packed.argtypes = [vp, C.POINTER(C.POINTER(C.c_int64)), C.POINTER(f64p), C.POINTER(f64p),
                                   C.POINTER(f64p), C.POINTER(f64p)]
    lib.bvp_get_packed.restype = C.c_int
    lib.bvp_eval_stage.argtypes = [vp, i32, i32, f64p, i32p, f64p, f64p] + [f64p] * 8
    lib.bvp_eval_stage.restype = C.c_int
    lib.bvp_dense_output.argtypes = [vp, i32, f64p, i32, f64p]
    lib.bvp_dense_output.restype = C.c_int
    f32p = C.POINTER(C.c_float)
    lib.bvp_mlp_create.argtypes = [i32, i32p, C.POINTER(vp)]
    lib.bvp_mlp_create.restype = C.c_int
    lib.bvp_mlp_num_params.argtypes = [vp]
    lib.bvp_mlp_num_params.restype = C.c_int64
    lib.bvp_mlp_set_params.argtypes = [vp, f32p]
    lib.bvp_mlp_set_params.restype = C.c_int
    lib.bvp_mlp_get_params.argtypes = [vp, f32p]
    lib.bvp_mlp_get_params.restype = C.c_int
    lib.bvp_mlp_set_normalization.argtypes = [vp, f32p, f32p, f32p, f32p]
    lib.bvp_mlp_set_normalization.restype = C.c_int
    lib.bvp_mlp_forward.argtypes = [vp, i32, f32p, f32p]
    lib.bvp_mlp_forward.restype = C.c_int
    lib.bvp_mlp_loss_grad.argtypes = [vp, i32, f32p, f32p, f32p, f32p]
    lib.bvp_mlp_loss_grad.restype = C.c_int
    lib.bvp_mlp_train.argtypes = [vp, i32, f32p, f32p, i32, i32, C.c_float, C.c_uint64, f32p]
    lib.bvp_mlp_train.restype = C.c_int
    lib.bvp_mlp_forward_device.argtypes = [vp, i32, vp, vp, vp]
    lib.bvp_mlp_forward_device.restype = C.c_int
    lib.bvp_mlp_forward_noalloc.argtypes = [vp, i32, vp, vp, vp]
    lib.bvp_mlp_forward_noalloc.restype = C.c_int
    lib.bvp_resample_guess_device.argtypes = [i32, i32, i32, vp, vp, vp, vp, vp, vp]
    lib.bvp_resample_guess_device.restype = C.c_int
    lib.bvp_mlp_destroy.argtypes = [vp]
    lib.bvp_mlp_destroy.restype = None
    lib.bvp_solve_batch_warm.argtypes = [vp, vp, i32, i32, f32p, i32, f64p, i32p, f64p, f64p,
                                         C.POINTER(Results), i32p]
    lib.bvp_solve_batch_warm.restype = C.c_int
    lib.bvp_solve_batch_device_warm.argtypes = [vp, vp, i32, vp, i32, vp, vp, vp, i32]
    lib.bvp_solve_batch_device_warm.restype = C.c_int
    lib.bvp_last_timing.argtypes = [vp, f64p]
    lib.bvp_last_timing.restype = C.c_int
    lib.bvp_get_tuning.argtypes = [vp, i32p]
    lib.bvp_get_tuning.restype = C.c_int
    lib.bvp_get_fused_tuning.argtypes = [vp, i32p, i32p, C.POINTER(C.c_float)]
    lib.bvp_get_fused_tuning.restype = C.c_int
    lib.bvp_get_block_mode.argtypes = [vp, i32p, i32p]
    lib.bvp_get_block_mode.restype = C.c_int
    lib.bvp_get_work_order.argtypes = [vp, i32p, C.POINTER(C.c_float), i32]
    lib.bvp_get_work_order.restype = C.c_int
    lib.bvp_stream.argtypes = [vp]
    lib.bvp_stream.restype = vp
    lib.bvp_last_error.argtypes = [vp]
    lib.bvp_last_error.restype = C.c_char_p
    lib.bvp_destroy.argtypes = [vp]
    lib.bvp_destroy.restype = None
    if path == LIB_PATH or _lib is None:
        _lib = lib
    return lib


def f64(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def i32(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None else None
