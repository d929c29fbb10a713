// Host runtime of libbvpgpu.so: the C ABI declared in include/bvpgpu.h.
//
// bvp_create JIT-compiles the device code (bvp_prelude.cuh + the user's problem source +
// bvp_kernels.cuh) with NVRTC for sm_103a, caches the cubin on disk, and loads it with
// the runtime's library API. bvp_solve_batch stages the inputs through pinned memory,
// launches the prep and the persistent fused solve kernels on the handle's stream, and
// brings the per-instance results and the packed solutions back.
//
// The host side of the reference path this replaces is SciMLBase.__init / solve! of
// lib/BoundaryValueDiffEqMIRK/src/mirk.jl:49-332 (setup, outer loop orchestration) and
// the EnsembleProblem loop over trajectories.
#include "bvpgpu.h"

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bvp_shared.h"
#include "bvp_firk_tableau.h"
#include "bvp_embedded.inc"  // kEmbedCount, kEmbedNames[], kEmbedSources[], kEmbedHash

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct HostBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct bvp_handle_s {
    bvp_problem_desc desc{};
    bvp_options opt{};
    std::string source;
    std::string err;
    BvpLayout L{};
    int js = 4;  // sizeof Jacobian scalar
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaLibrary_t lib = nullptr;
    cudaKernel_t k_fused = nullptr, k_stage = nullptr, k_pack = nullptr, k_probe = nullptr, k_offsets = nullptr,
                 k_convert = nullptr, k_prep = nullptr, k_dense = nullptr, k_learn = nullptr;
    // work-order autotuner of the fused solve: the first solves of at least kLearnMin instances
    // record every instance's solve time; bvp_learn_costs folds them into a cost table per
    // initial-size bucket, and bvp_prep orders later solves longest first from it
    DevBuf d_inst_cost, d_cost_tab;
    int learn_left = 3;
    bool have_tab = false;
    // launch-shape autotuner of the fused solve: the kernel built for 4, 3 and 2 resident
    // blocks per SM; once the work order is learned, the next solves of one batch shape rotate
    // through the three (an untimed first launch, then two timed solves each) and the handle
    // keeps the fastest
    cudaKernel_t k_fused_v[3] = {nullptr, nullptr, nullptr};
    int occ_v[3] = {4, 3, 2}, occ_hi = 3;   // resident blocks per SM of each fused kernel
    int group_min = 0;   // meshes of at least this many intervals are solved in block mode (0: none)
    // the block-mode module (BVP_BLOCK_MODE), built on the first batch that has a long mesh
    cudaLibrary_t lib_blk = nullptr;
    cudaKernel_t k_fused_blk = nullptr;
    int occ_blk = 2;
    bool last_blk = false;   // the last solve ran the block-mode module
    int fused_pick = 1;
    struct {
        long long key = -1;
        int pending = -1, next = 0;
        float sum[3] = {0, 0, 0};
        int cnt[3] = {0, 0, 0};
        bool seen[3] = {false, false, false};   // a candidate's first launch (module load) is not timed
        bool done = false;
    } tune;
    // error controllers other than DefectControl (fused path): the global estimates per interval,
    // and for HOErrorControl the module compiled for MIRK(p+2), its stage array, the two lists
    // of instances waiting for its solve and their counts (pinned for the host's loop)
    bool glob = false, ho = false;
    // a FIRK scheme (options.firk): its coefficients, the stage unknowns and condensation
    // record per interval, and the records' array
    bool firk = false;
    BvpFirkTab ftab{};
    int firk_fn = 0, firk_fxw = 0;
    DevBuf d_fx;
    BvpLayout L_hi{};
    cudaLibrary_t lib_hi = nullptr;
    cudaKernel_t k_fused_hi = nullptr, k_probe_hi = nullptr;
    DevBuf d_gerr, d_K_hi, d_pause;
    HostBuf h_pause;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    // the surrogate's forward of a warm solve runs on a second stream, beside the solve's
    // per-batch setup; the fused kernel waits for it on ev_side
    cudaStream_t side = nullptr;
    cudaEvent_t ev_in = nullptr, ev_side = nullptr;
    // larger-state path (M > 8, bvp_large.cuh)
    bool large = false;
    cudaKernel_t kl_res = nullptr, kl_jac = nullptr, kl_solve = nullptr, kl_update = nullptr, kl_copy = nullptr,
                 kl_defect = nullptr, kl_transfer = nullptr, kl_convert = nullptr, kl_probe = nullptr,
                 kl_dense = nullptr, kl_scatter = nullptr;
    BvpLargeArgs la{};       // the last larger-state solve's arguments (dense output reads them)
    int l_threads = 256;     // bl_linsolve block size, picked by large_tune_linsolve
    size_t l_smem = 0;
    size_t l_warp_bytes = 0, l_dense_bytes = 0;
    bool l_tuned = false;
    size_t j_warp_bytes = 0; // bl_jacobian: shared memory per warp, and the parameter staging limit
    int j_pmax = 0;
    DevBuf d_bcres, d_G, d_lnorm, d_lsq, d_ldnorm, d_lbad, d_active, d_N, d_newN;
    // device arrays
    DevBuf d_mesh, d_h, d_y, d_ybak, d_ybase, d_K, d_KI, d_F, d_err, d_inc, d_iold, d_Sb, d_Rb,
        d_rec, d_tj, d_hj, d_delta, d_yj, d_Fj, d_scr, d_iscr, d_st, d_order, d_cap, d_node_off, d_counter,
        d_params, d_params_j, d_n_init, d_tspans, d_y0, d_y0_off, d_out_off, d_out_mesh,
        d_out_y, d_out_K, d_out_KI, d_norm, d_feat, d_grid;
    // pinned host staging
    HostBuf h_in, h_st, h_off, h_mesh, h_y, h_K, h_KI;
    long long out_cap = 0;   // points the packed host outputs hold
    // last batch
    int last_n = 0;
    long long last_tot = 0;
    bool have_results = false;
    bool pending_device = false;
    bool stages_ok = false;  // K and KI on the device belong to the last batch
    int pending_n = 0;
    double timing_ms[2] = {0, 0};
    std::vector<BvpInstState> st;
    std::vector<int64_t> offsets;
};

namespace {

bvp_status fail(bvp_handle* h, bvp_status s, const std::string& msg) {
    if (h) h->err = msg;
    return s;
}

#define CU(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(h, BVP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

bool ensure_dev(DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (cudaMalloc(&b.p, bytes) != cudaSuccess) { b.p = nullptr; return false; }
    b.bytes = bytes;
    return true;
}

bool ensure_host(HostBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return true;
    if (b.p) cudaFreeHost(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (cudaMallocHost(&b.p, bytes) != cudaSuccess) { b.p = nullptr; return false; }
    b.bytes = bytes;
    return true;
}

uint64_t fnv1a(const void* data, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}

std::string lib_dir() {
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&bvp_default_options), &info) && info.dli_fname) {
        std::string p(info.dli_fname);
        const size_t k = p.rfind('/');
        if (k != std::string::npos) return p.substr(0, k);
    }
    return ".";
}

std::string cache_dir() {
    const char* env = std::getenv("BVPGPU_CACHE_DIR");
    std::string d = env && *env ? std::string(env) : lib_dir() + "/jit_cache";
    mkdir(d.c_str(), 0755);
    return d;
}

bool read_file(const std::string& path, std::vector<char>& out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out.resize(n > 0 ? size_t(n) : 0);
    const size_t got = n > 0 ? std::fread(out.data(), 1, size_t(n), f) : 0;
    std::fclose(f);
    return n > 0 && got == size_t(n);
}

void write_file_atomic(const std::string& path, const std::vector<char>& data) {
    const std::string tmp = path + ".tmp" + std::to_string(long(getpid()));
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;
    std::fwrite(data.data(), 1, data.size(), f);
    std::fclose(f);
    std::rename(tmp.c_str(), path.c_str());
}

}  // namespace

extern "C" {

void bvp_default_options(bvp_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->order = 4;
    o->adaptive = 1;
    o->max_subintervals = 3000;
    o->max_newton = 100;
    o->max_rounds = 64;
    o->transfer_inplace = 1;
    o->bc_jac_exact = 0;
    o->linesearch_fallback = 1;
    o->stall_steps = 32;
    o->jac_precision = 32;
    o->want_stages = 0;
    o->fp32_phase = 1;
    o->abstol = 1e-6;
    o->defect_threshold = 0.1;
    o->divergence_factor = 1e3;
    o->mirk6i = 0;
    o->controller = BVP_CTL_DEFECT;
    o->global_method = BVP_GLOBAL_HO;
    o->hybrid_de = 1.0;
    o->hybrid_ge = 1.0;
}

const char* bvp_last_error(bvp_handle* h) { return h ? h->err.c_str() : "null handle"; }

void* bvp_stream(bvp_handle* h) { return h ? static_cast<void*>(h->stream) : nullptr; }

// NVRTC build of the problem's module for one MIRK order (the cubin is cached on disk under a
// hash of the sources and options). global_ctl compiles in the error controllers other than
// DefectControl.
static bvp_status build_cubin(bvp_handle* h, int order, int mirk6i, int global_ctl, std::vector<char>& cubin,
                              const std::string& prefix = std::string()) {
    const bvp_problem_desc& d = h->desc;
    const bvp_options& o = h->opt;
    std::vector<std::string> opts = {
        "--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "--fmad=true",
        "-DBVP_M=" + std::to_string(d.M), "-DBVP_ORDER=" + std::to_string(order),
        "-DBVP_TWOPOINT=" + std::to_string(d.twopoint),
        "-DBVP_NBC=" + std::to_string(d.twopoint ? 2 : d.n_bc_pts),
        "-DBVP_LA=" + std::to_string(d.twopoint ? d.La : 0),
        std::string("-DBVP_JT=") + (o.jac_precision == 64 ? "double" : "float"),
        std::string("-DBVP_MIRK6I=") + (mirk6i ? "1" : "0"),
        // a source with BVP_SING has a singular term S y / t (the problem's singular_term)
        std::string("-DBVP_SINGULAR=") + (h->source.find("BVP_SING") != std::string::npos ? "1" : "0"),
    };
    if (global_ctl) opts.push_back("-DBVP_GLOBAL_CTL=1");
    const bool large = d.M > 8;
    const std::string src = std::string("#include \"bvp_prelude.cuh\"\n") + prefix + "#line 1 \"problem_source\"\n" +
                            h->source + (large ? "\n#include \"bvp_large.cuh\"\n" : "\n#include \"bvp_kernels.cuh\"\n");
    uint64_t key = fnv1a(kEmbedHash, std::strlen(kEmbedHash));
    key = fnv1a(src.data(), src.size(), key);
    for (auto& s : opts) key = fnv1a(s.data(), s.size() + 1, key);
    char name[64];
    std::snprintf(name, sizeof(name), "/bvp_%016llx.cubin", (unsigned long long)key);
    const std::string path = cache_dir() + name;
    if (!read_file(path, cubin)) {
        nvrtcProgram prog;
        if (nvrtcCreateProgram(&prog, src.c_str(), "bvp_problem.cu", kEmbedCount, kEmbedSources,
                               kEmbedNames) != NVRTC_SUCCESS)
            return fail(h, BVP_ERR_COMPILE, "nvrtcCreateProgram failed");
        std::vector<const char*> cop;
        for (auto& s : opts) cop.push_back(s.c_str());
        const nvrtcResult rc = nvrtcCompileProgram(prog, int(cop.size()), cop.data());
        size_t logn = 0;
        nvrtcGetProgramLogSize(prog, &logn);
        std::string log(logn, '\0');
        if (logn) nvrtcGetProgramLog(prog, &log[0]);
        if (rc != NVRTC_SUCCESS) {
            nvrtcDestroyProgram(&prog);
            return fail(h, BVP_ERR_COMPILE, "NVRTC: " + std::string(nvrtcGetErrorString(rc)) + "\n" + log);
        }
        size_t n = 0;
        nvrtcGetCUBINSize(prog, &n);
        cubin.resize(n);
        nvrtcGetCUBIN(prog, cubin.data());
        nvrtcDestroyProgram(&prog);
        write_file_atomic(path, cubin);
    }
    return BVP_OK;
}

// Meshes of at least this many initial intervals are solved by a whole block (block mode:
// the residuals and defects over 128 lanes) unless bvp_options.block_min says otherwise.
static constexpr int kGroupMinDefault = 512;

// Resident 128-thread blocks per SM of a loaded kernel (registers and shared memory), or the
// fallback when the runtime cannot say.
static int kernel_occupancy(cudaKernel_t k, int fallback) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k, 128, 0) != cudaSuccess || nb <= 0) {
        (void)cudaGetLastError();
        return fallback;
    }
    return nb;
}

static bvp_status compile_and_load(bvp_handle* h) {
    const bool large = h->desc.M > 8;
    std::vector<char> cubin;
    // a FIRK handle's module: the MIRK4 build with the FIRK scheme's constants and solve path
    bvp_status bs = h->firk ? build_cubin(h, 4, 0, 0, cubin, bvp_firk_constants(h->ftab))
                            : build_cubin(h, h->opt.order, h->opt.mirk6i, h->glob ? 1 : 0, cubin);
    if (bs != BVP_OK) return bs;
    CU(cudaLibraryLoadData(&h->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    if (large) {
        h->large = true;
        CU(cudaLibraryGetKernel(&h->kl_res, h->lib, "bl_residual"));
        CU(cudaLibraryGetKernel(&h->kl_jac, h->lib, "bl_jacobian"));
        CU(cudaLibraryGetKernel(&h->kl_solve, h->lib, "bl_linsolve"));
        CU(cudaLibraryGetKernel(&h->kl_update, h->lib, "bl_update"));
        CU(cudaLibraryGetKernel(&h->kl_copy, h->lib, "bl_copy"));
        CU(cudaLibraryGetKernel(&h->kl_defect, h->lib, "bl_defect"));
        CU(cudaLibraryGetKernel(&h->kl_transfer, h->lib, "bl_transfer"));
        CU(cudaLibraryGetKernel(&h->kl_convert, h->lib, "bl_convert_params"));
        CU(cudaLibraryGetKernel(&h->kl_probe, h->lib, "bl_layout_probe"));
        CU(cudaLibraryGetKernel(&h->kl_dense, h->lib, "bl_dense"));
        CU(cudaLibraryGetKernel(&h->kl_scatter, h->lib, "bl_scatter"));
        return BVP_OK;
    }
    CU(cudaLibraryGetKernel(&h->k_fused, h->lib, "bvp_solve_fused"));
    h->k_fused_v[0] = h->k_fused;
    if (h->glob || h->firk) {
        // one fused kernel in these builds: nothing to tune
        h->k_fused_v[1] = h->k_fused_v[2] = h->k_fused;
        h->fused_pick = 1;
        h->tune.done = true;
    } else {
        CU(cudaLibraryGetKernel(&h->k_fused_v[1], h->lib, "bvp_solve_fused_b3"));
        CU(cudaLibraryGetKernel(&h->k_fused_v[2], h->lib, "bvp_solve_fused_b2"));
    }
    for (int v = 0; v < 3; ++v) h->occ_v[v] = kernel_occupancy(h->k_fused_v[v], h->occ_v[v]);
    // block mode for long meshes, in the defect-controlled MIRK build
    if (!h->glob && !h->firk)
        h->group_min = h->opt.block_min == 0 ? kGroupMinDefault : std::max(0, h->opt.block_min);
    if (!h->firk) CU(cudaLibraryGetKernel(&h->k_stage, h->lib, "bvp_stage"));
    CU(cudaLibraryGetKernel(&h->k_pack, h->lib, "bvp_pack"));
    CU(cudaLibraryGetKernel(&h->k_offsets, h->lib, "bvp_out_offsets"));
    CU(cudaLibraryGetKernel(&h->k_probe, h->lib, "bvp_layout_probe"));
    CU(cudaLibraryGetKernel(&h->k_convert, h->lib, "bvp_convert_params"));
    CU(cudaLibraryGetKernel(&h->k_prep, h->lib, "bvp_prep"));
    if (!h->firk) CU(cudaLibraryGetKernel(&h->k_dense, h->lib, "bvp_dense"));
    CU(cudaLibraryGetKernel(&h->k_learn, h->lib, "bvp_learn_costs"));
    if (h->ho) {
        // HOErrorControl's second solve: the same problem with MIRK(p+2) (adaptivity.jl:552-555)
        std::vector<char> cubin_hi;
        bs = build_cubin(h, h->opt.order + 2, 0, 1, cubin_hi, "#define BVP_POLISH_ONLY 1\n");
        if (bs != BVP_OK) return bs;
        CU(cudaLibraryLoadData(&h->lib_hi, cubin_hi.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
        CU(cudaLibraryGetKernel(&h->k_fused_hi, h->lib_hi, "bvp_solve_fused"));
        CU(cudaLibraryGetKernel(&h->k_probe_hi, h->lib_hi, "bvp_layout_probe"));
        h->occ_hi = kernel_occupancy(h->k_fused_hi, h->occ_hi);
    }
    return BVP_OK;
}

static size_t large_jac_smem(const bvp_handle* h);

bvp_status bvp_create(const bvp_problem_desc* desc, const char* source, const bvp_options* opt,
                      bvp_handle** out) {
    bvp_handle* h = nullptr;
    if (!desc || !source || !out) return BVP_ERR_INVALID;
    *out = nullptr;
    h = new bvp_handle_s();
    h->desc = *desc;
    if (opt) h->opt = *opt; else bvp_default_options(&h->opt);
    h->source = source;
    const bvp_problem_desc& d = h->desc;
    const bvp_options& o = h->opt;
    std::string why;
    if (d.M < 1 || d.M > 32) why = "M must be in 1..32";
    else if (d.M > 8 && !d.twopoint) why = "M > 8 takes two-point boundary conditions";
    else if (d.n_params < 0) why = "n_params must be >= 0";
    else if (!d.twopoint && (d.n_bc_pts < 1 || d.n_bc_pts > 16)) why = "n_bc_pts must be in 1..16";
    else if (d.twopoint && (d.La < 0 || d.Lb < 0 || d.La + d.Lb != d.M)) why = "La + Lb must equal M";
    else if (o.order < 2 || o.order > 6) why = "order must be 2..6";
    else if (o.mirk6i != 0 && (o.mirk6i != 1 || o.order != 6)) why = "mirk6i takes order 6";
    else if (!(o.abstol > 0)) why = "abstol must be > 0";
    else if (o.max_subintervals < 1) why = "max_subintervals must be >= 1";
    else if (o.jac_precision != 32 && o.jac_precision != 64) why = "jac_precision must be 32 or 64";
    else if (o.controller < BVP_CTL_DEFECT || o.controller > BVP_CTL_HYBRID) why = "controller must be 0..3";
    else if (o.global_method != BVP_GLOBAL_HO && o.global_method != BVP_GLOBAL_RE) why = "global_method must be 0 or 1";
    else if (o.controller != BVP_CTL_DEFECT && d.M > 8) why = "error controllers other than DefectControl take M <= 8";
    else if (o.controller != BVP_CTL_DEFECT && o.global_method == BVP_GLOBAL_HO && (o.order + 2 > 6 || o.mirk6i))
        why = "HOErrorControl solves with MIRK(order + 2): orders 2, 3 and 4";
    else if (o.firk < 0 || o.firk > 4) why = "firk must be 0..4";
    else if (o.firk && bvp_firk_tableau(o.firk, o.firk_stages).order == 0) why = "no such FIRK scheme";
    else if (o.firk && (d.M > 8 || o.firk_stages * d.M > 32 || o.controller != BVP_CTL_DEFECT || o.want_stages ||
                        h->source.find("BVP_SING") != std::string::npos))
        why = "the FIRK path takes M <= 8, stages x M <= 32, DefectControl, no stage output and no singular term";
    else if (o.firk && o.adaptive &&
             ((o.firk == 1 && o.firk_stages == 1) || ((o.firk == 3 || o.firk == 4) && o.firk_stages == 2)))
        why = "RadauIIa1, LobattoIIIb2 and LobattoIIIc2 have no adaptivity (algorithms.jl:411)";
    if (!why.empty()) { delete h; return BVP_ERR_INVALID; }
    if (o.firk) {
        // FP64 throughout: the stage unknowns and their condensation in the Jacobian precision
        h->firk = true;
        h->ftab = bvp_firk_tableau(o.firk, o.firk_stages);
        h->firk_fn = o.firk_stages * d.M;
        h->firk_fxw = h->firk_fn * (d.M + 1);
        h->opt.jac_precision = 64;
        h->opt.fp32_phase = 0;
        h->opt.linesearch_fallback = 0;
    }
    h->L = bvp_make_layout(d.M, h->firk ? 4 : o.order, d.twopoint ? 2 : d.n_bc_pts, d.twopoint, h->firk ? 0 : o.mirk6i);
    h->glob = o.adaptive && o.controller != BVP_CTL_DEFECT;
    h->ho = h->glob && o.global_method == BVP_GLOBAL_HO;
    if (h->ho) h->L_hi = bvp_make_layout(d.M, o.order + 2, d.twopoint ? 2 : d.n_bc_pts, d.twopoint, 0);
    h->js = h->opt.jac_precision == 64 ? 8 : 4;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaEventCreate(&h->ev[k]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_side, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        h->err = std::string("CUDA init: ") + cudaGetErrorString(e);
        *out = h;
        return BVP_ERR_CUDA;
    }
    bvp_status s = compile_and_load(h);
    *out = h;
    if (s != BVP_OK) return s;
    if (h->large) {
        // host/device launch ABI of the larger-state kernels, and their shared memory
        DevBuf probe;
        if (!ensure_dev(probe, 16 * sizeof(int))) return fail(h, BVP_ERR_NOMEM, "probe alloc");
        int* pp = static_cast<int*>(probe.p);
        void* args[] = {&pp};
        CU(cudaLaunchKernel((const void*)h->kl_probe, dim3(1), dim3(1), args, 0, h->stream));
        int got[16] = {0};
        CU(cudaMemcpyAsync(got, probe.p, sizeof(got), cudaMemcpyDeviceToHost, h->stream));
        CU(cudaStreamSynchronize(h->stream));
        cudaFree(probe.p);
        if (got[0] != int(sizeof(BvpLargeArgs)) || got[1] != h->L.RECW || got[4] != h->L.S || got[5] != h->L.NSXA)
            return fail(h, BVP_ERR_STATE, "host/device layout mismatch (larger-state kernels)");
        // per warp: relation, panel factors, pivot indices and the staged block; plus the
        // dense end system. Up to 8 warps as fit in the SM's shared memory; the block size is
        // tuned on the first solve (large_tune_linsolve).
        h->l_warp_bytes = size_t(got[2]);
        h->l_dense_bytes = size_t(got[6]);
        int max_smem = 0, dev = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        int wmax = int((size_t(max_smem) - h->l_dense_bytes) / h->l_warp_bytes);
        wmax = std::min(wmax, 8);
        if (wmax < 3) return fail(h, BVP_ERR_STATE, "larger-state linear solve: shared memory too small");
        h->l_threads = 32 * wmax;
        h->l_smem = size_t(wmax) * h->l_warp_bytes + h->l_dense_bytes;
        CU(cudaFuncSetAttribute((const void*)h->kl_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, int(h->l_smem)));
        h->j_warp_bytes = size_t(got[3]);
        h->j_pmax = got[7];
        CU(cudaFuncSetAttribute((const void*)h->kl_jac, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(large_jac_smem(h))));
        return BVP_OK;
    }
    // check that host and device agree on the launch ABI
    DevBuf probe;
    if (!ensure_dev(probe, 16 * sizeof(int))) return fail(h, BVP_ERR_NOMEM, "probe alloc");
    int* pp = static_cast<int*>(probe.p);
    void* args[] = {&pp};
    CU(cudaLaunchKernel((const void*)h->k_probe, dim3(1), dim3(1), args, 0, h->stream));
    int got[16] = {0};
    CU(cudaMemcpyAsync(got, probe.p, sizeof(got), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    cudaFree(probe.p);
    const BvpLayout& L = h->L;
    if (got[0] != L.SCRW || got[1] != L.ISCRW || got[2] != L.EQW || got[3] != L.RECW ||
        got[4] != int(sizeof(BvpArgs)) || got[5] != int(sizeof(BvpInstState)) ||
        got[6] != L.NSXA || got[7] != L.S)
        return fail(h, BVP_ERR_STATE, "host/device layout mismatch");
    if (h->ho) {
        DevBuf probe2;
        if (!ensure_dev(probe2, 16 * sizeof(int))) return fail(h, BVP_ERR_NOMEM, "probe alloc");
        int* p2 = static_cast<int*>(probe2.p);
        void* args2[] = {&p2};
        CU(cudaLaunchKernel((const void*)h->k_probe_hi, dim3(1), dim3(1), args2, 0, h->stream));
        int got2[16] = {0};
        CU(cudaMemcpyAsync(got2, probe2.p, sizeof(got2), cudaMemcpyDeviceToHost, h->stream));
        CU(cudaStreamSynchronize(h->stream));
        cudaFree(probe2.p);
        const BvpLayout& H = h->L_hi;
        if (got2[0] != H.SCRW || got2[1] != H.ISCRW || got2[4] != int(sizeof(BvpArgs)) ||
            got2[5] != int(sizeof(BvpInstState)) || got2[7] != H.S)
            return fail(h, BVP_ERR_STATE, "host/device layout mismatch (MIRK(p+2) module)");
    }
    return BVP_OK;
}

static bvp_status ensure_arena(bvp_handle* h, long long tot, int n, long long y0_vals) {
    const BvpLayout& L = h->L;
    const int M = L.M, js = h->js;
    const size_t T = size_t(tot);
    bool ok = ensure_dev(h->d_mesh, 2 * T * 8) && ensure_dev(h->d_h, 2 * T * 8) &&
              ensure_dev(h->d_y, 2 * T * M * 8) && ensure_dev(h->d_ybak, T * M * 8) &&
              ensure_dev(h->d_ybase, T * M * 8) && ensure_dev(h->d_K, T * std::max(L.S * M, h->firk_fn) * 8) &&
              ensure_dev(h->d_KI, T * L.NSXA * M * 8) && ensure_dev(h->d_F, T * M * 8) &&
              ensure_dev(h->d_err, T * 8) && ensure_dev(h->d_inc, T * M * 8) &&
              ensure_dev(h->d_iold, T * 4) && ensure_dev(h->d_Sb, T * M * M * js) &&
              ensure_dev(h->d_Rb, T * M * M * js) && ensure_dev(h->d_rec, T * L.RECW * js) &&
              ensure_dev(h->d_delta, T * M * js) &&
              ensure_dev(h->d_yj, T * M * js) && ensure_dev(h->d_Fj, T * M * js) &&
              ensure_dev(h->d_tj, T * js) && ensure_dev(h->d_hj, T * js) &&
              ensure_dev(h->d_scr, size_t(n) * std::max(L.SCRW, h->ho ? h->L_hi.SCRW : 0) * 8) &&
              ensure_dev(h->d_iscr, size_t(n) * L.ISCRW * 4) &&
              ensure_dev(h->d_st, size_t(n) * sizeof(BvpInstState)) && ensure_dev(h->d_order, size_t(n) * 4) &&
              ensure_dev(h->d_cap, size_t(n) * 4) && ensure_dev(h->d_node_off, size_t(n) * 8) &&
              ensure_dev(h->d_counter, 32) &&
              ensure_dev(h->d_params, size_t(n) * std::max(1, h->desc.n_params) * 8) &&
              ensure_dev(h->d_params_j, size_t(n) * std::max(1, h->desc.n_params) * js) &&
              ensure_dev(h->d_n_init, size_t(n) * 4) && ensure_dev(h->d_tspans, size_t(n) * 16) &&
              ensure_dev(h->d_y0, size_t(std::max<long long>(y0_vals, 1)) * 8) &&
              ensure_dev(h->d_y0_off, size_t(n + 1) * 8) && ensure_dev(h->d_out_off, size_t(n + 1) * 8) &&
              ensure_dev(h->d_norm, size_t(n) * 8);
    if (ok && h->glob) ok = ensure_dev(h->d_gerr, T * 8);
    if (ok && h->firk) ok = ensure_dev(h->d_fx, T * h->firk_fxw * 8);
    if (ok && h->ho)
        ok = ensure_dev(h->d_K_hi, T * h->L_hi.S * M * 8) && ensure_dev(h->d_pause, (size_t(2) * n + 2) * 4) &&
             ensure_host(h->h_pause, 16);
    if (!ok) return fail(h, BVP_ERR_NOMEM, "device allocation failed");
    return BVP_OK;
}

static void fill_args(bvp_handle* h, BvpArgs& a, int n, long long tot, int y0_mode, const double* d_params,
                      const int* d_n_init, const double* d_tspans, const double* d_y0, const long long* d_y0_off) {
    const bvp_options& o = h->opt;
    std::memset(&a, 0, sizeof(a));
    a.n_inst = n;
    a.n_params = h->desc.n_params;
    a.adaptive = o.adaptive;
    a.max_sub = o.max_subintervals;
    a.max_newton = o.max_newton;
    a.max_rounds = o.max_rounds;
    a.stall_steps = o.stall_steps;
    a.transfer_inplace = o.transfer_inplace;
    a.bc_jac_exact = o.bc_jac_exact;
    a.linesearch = o.linesearch_fallback;
    a.want_stages = o.want_stages;
    a.y0_mode = y0_mode;
    a.fp32_phase = (o.fp32_phase && o.jac_precision == 32) ? 1 : 0;
    a.abstol = o.abstol;
    a.defect_threshold = o.defect_threshold;
    a.divergence_factor = o.divergence_factor;
    for (int k = 0; k < 16; ++k) a.bc_t[k] = h->desc.bc_t[k];
    a.tot = tot;
    a.order = static_cast<const int*>(h->d_order.p);
    a.work_counter = static_cast<int*>(h->d_counter.p);
    a.deal_sms = 0;
    a.params = d_params;
    a.params_j = h->d_params_j.p;
    a.n_init = d_n_init;
    a.tspans = d_tspans;
    a.y0 = d_y0;
    a.y0_off = d_y0_off;
    a.node_off = static_cast<const bvp_i64*>(h->d_node_off.p);
    a.cap = static_cast<const int*>(h->d_cap.p);
    a.mesh = static_cast<double*>(h->d_mesh.p);
    a.h = static_cast<double*>(h->d_h.p);
    a.y = static_cast<double*>(h->d_y.p);
    a.ybak = static_cast<double*>(h->d_ybak.p);
    a.ybase = static_cast<double*>(h->d_ybase.p);
    a.K = static_cast<double*>(h->d_K.p);
    a.KI = static_cast<double*>(h->d_KI.p);
    a.F = static_cast<double*>(h->d_F.p);
    a.err = static_cast<double*>(h->d_err.p);
    a.inc = static_cast<double*>(h->d_inc.p);
    a.iold = static_cast<int*>(h->d_iold.p);
    a.Sb = h->d_Sb.p;
    a.Rb = h->d_Rb.p;
    a.rec = h->d_rec.p;
    a.delta = h->d_delta.p;
    a.yj = h->d_yj.p;
    a.Fj = h->d_Fj.p;
    a.tj = h->d_tj.p;
    a.hj = h->d_hj.p;
    a.scr = static_cast<double*>(h->d_scr.p);
    a.iscr = static_cast<int*>(h->d_iscr.p);
    a.st = static_cast<BvpInstState*>(h->d_st.p);
    a.controller = h->glob ? o.controller : BVP_CTL_DEFECT;
    a.global_method = o.global_method;
    a.hybrid_de = o.hybrid_de;
    a.hybrid_ge = o.hybrid_ge;
    a.gerr = static_cast<double*>(h->d_gerr.p);
    a.fx = static_cast<double*>(h->d_fx.p);
    a.phase = 0;
    if (h->ho) {
        a.pause_count = static_cast<int*>(h->d_pause.p);
        a.pause_list = a.pause_count + 2;
    }
}

// Node capacity of an instance: room for max(n, max_subintervals) intervals, twice that when
// REErrorControl solves on the halved mesh.
static int cap_scale(const bvp_handle* h) { return (h->glob && h->opt.global_method == BVP_GLOBAL_RE) ? 2 : 1; }
static long long cap_nodes(const bvp_handle* h, long long ni) {
    return cap_scale(h) * std::max<long long>(ni, h->opt.max_subintervals) + 1;
}

// A fused kernel's grid for the static deal (BvpArgs::deal_sms): a whole number of blocks per
// SM, no more than the SMs hold at once (so every block starts together), and no more rounds
// of blocks than the batch fills.
static int resident_grid(bvp_handle* h, int n, int occ) {
    const int sms = std::max(1, h->sm_count);
    const int rounds = std::max(1, std::min(std::max(1, occ), (n + 4 * sms - 1) / (4 * sms)));
    return rounds * sms;
}

static int fused_grid(bvp_handle* h, int n) {
    const int warps_per_block = 4;
    const int want = (n + warps_per_block - 1) / warps_per_block;
    const int cap = std::max(1, h->sm_count) * 16;
    return std::max(1, std::min(want, cap));
}

// Launches prep + conversion + fused solve on the handle's stream.
static bvp_status prepare_host_outputs(bvp_handle* h, int n, long long pts_guess, BvpArgs& a);

static constexpr int kLearnMin = 256;   // smallest batch the work-order autotuner learns from
static constexpr int kFusedBlocks[3] = {4, 3, 2};   // resident blocks per SM of the fused variants

// The fused variant for the next launch. Folds the previous launch's kernel time into the
// launch-shape tuner when that launch ran a candidate and has completed; candidates are
// compared on one batch shape (instance count, guess form) after the work order is learned.
static int fused_variant(bvp_handle* h, int n, int y0_mode) {
    auto& t = h->tune;
    if (t.done || h->ho) return h->fused_pick;
    if (t.pending >= 0) {
        float ms = 0.0f;
        if (cudaEventQuery(h->ev[2]) == cudaSuccess && cudaEventElapsedTime(&ms, h->ev[1], h->ev[2]) == cudaSuccess) {
            t.sum[t.pending] += ms;
            ++t.cnt[t.pending];
        } else {
            (void)cudaGetLastError();   // not ready: that sample is dropped
        }
        t.pending = -1;
    }
    if (t.cnt[0] >= 2 && t.cnt[1] >= 2 && t.cnt[2] >= 2) {
        int best = 0;
        for (int c = 1; c < 3; ++c)
            if (t.sum[c] / t.cnt[c] < t.sum[best] / t.cnt[best]) best = c;
        h->fused_pick = best;
        t.done = true;
        return best;
    }
    if (n < kLearnMin || h->learn_left > 0) return h->fused_pick;
    const long long key = (long long)n * 4 + y0_mode;
    if (key != t.key) {
        t.key = key;
        t.next = 0;
        for (int c = 0; c < 3; ++c) { t.sum[c] = 0.0f; t.cnt[c] = 0; }
    }
    const int c = t.next;
    t.next = (t.next + 1) % 3;
    if (t.seen[c]) t.pending = c;
    t.seen[c] = true;
    return c;
}

// HOErrorControl: instances stop after each round's Newton solve (and defect) and wait in a list
// for their MIRK(p+2) solve on the same mesh, which the module of that order runs (phase 2, its
// own stage array, the solution arrays shared); the solve's module then resumes them (phase 1)
// from the global estimate to the next round, where they may stop again. One host
// synchronisation per mesh round reads how many stopped.
static bvp_status ho_rounds(bvp_handle* h, const BvpArgs& a0, int n) {
    int* cnt = static_cast<int*>(h->d_pause.p);
    int* lists[2] = {cnt + 2, cnt + 2 + n};
    int* hc = static_cast<int*>(h->h_pause.p);
    int cur = 0;
    for (int round = 0; round <= h->opt.max_rounds + 1; ++round) {
        CU(cudaMemcpyAsync(hc, cnt + cur, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        CU(cudaStreamSynchronize(h->stream));
        const int c = *hc;
        if (c <= 0) return BVP_OK;
        if (c > n) return fail(h, BVP_ERR_STATE, "pause list overflow");
        BvpArgs a2 = a0;
        a2.phase = 2;
        a2.n_inst = c;
        a2.order = lists[cur];
        a2.K = static_cast<double*>(h->d_K_hi.p);
        a2.inst_cost = nullptr;
        a2.host_mesh = nullptr;
        CU(cudaMemsetAsync(a0.work_counter, 0, sizeof(int), h->stream));
        {
            void* args[] = {&a2};
            CU(cudaLaunchKernel((const void*)h->k_fused_hi, dim3(resident_grid(h, c, h->occ_hi)), dim3(128), args, 0,
                                h->stream));
        }
        BvpArgs a1 = a0;
        a1.phase = 1;
        a1.n_inst = c;
        a1.order = lists[cur];
        a1.pause_list = lists[cur ^ 1];
        a1.pause_count = cnt + (cur ^ 1);
        a1.inst_cost = nullptr;
        CU(cudaMemsetAsync(a0.work_counter, 0, sizeof(int), h->stream));
        CU(cudaMemsetAsync(a1.pause_count, 0, sizeof(int), h->stream));
        {
            void* args[] = {&a1};
            CU(cudaLaunchKernel((const void*)h->k_fused_v[h->fused_pick],
                                dim3(resident_grid(h, c, h->occ_v[h->fused_pick])), dim3(128), args, 0, h->stream));
        }
        cur ^= 1;
    }
    return fail(h, BVP_ERR_STATE, "HOErrorControl rounds did not end");
}

// The block-mode module: the same sources with BVP_BLOCK_MODE, one fused kernel. Built (or read
// from the cubin cache) when a batch first has a mesh of group_min intervals or more.
static bvp_status ensure_block_module(bvp_handle* h) {
    if (h->k_fused_blk) return BVP_OK;
    std::vector<char> cubin;
    bvp_status bs = build_cubin(h, h->opt.order, h->opt.mirk6i, 0, cubin, "#define BVP_BLOCK_MODE 1\n");
    if (bs != BVP_OK) return bs;
    CU(cudaLibraryLoadData(&h->lib_blk, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    CU(cudaLibraryGetKernel(&h->k_fused_blk, h->lib_blk, "bvp_solve_fused"));
    h->occ_blk = kernel_occupancy(h->k_fused_blk, 2);
    return BVP_OK;
}

static bvp_status launch_solve(bvp_handle* h, int n, long long tot, int y0_mode, const double* d_params,
                               const int* d_n_init, const double* d_tspans, const double* d_y0,
                               const long long* d_y0_off, int max_init, const float* d_grid = nullptr,
                               int n_grid = 0, long long host_pts = 0, bool wait_side = false) {
    // block mode when the batch has a long mesh (max_init: its largest initial interval count)
    bool blk = h->group_min > 0 && max_init >= h->group_min;
    if (blk && ensure_block_module(h) != BVP_OK) {
        // block mode only changes speed: without its module the handle solves by warps (the
        // reason stays in bvp_last_error)
        (void)cudaGetLastError();
        h->group_min = 0;
        blk = false;
    }
    h->last_blk = blk;
    BvpArgs a;
    fill_args(h, a, n, tot, y0_mode, d_params, d_n_init, d_tspans, d_y0, d_y0_off);
    a.y0_grid = d_grid;
    a.n_grid = n_grid;
    // the learned order times whole solves; with the MIRK(p+2) solves between launches it is not learned
    const bool learn = h->learn_left > 0 && n >= kLearnMin && !h->ho;
    if (learn) {
        if (!h->d_cost_tab.p) {
            if (!ensure_dev(h->d_cost_tab, (BVP_COST_BUCKETS + 1) * sizeof(float)))
                return fail(h, BVP_ERR_NOMEM, "cost table allocation failed");
            CU(cudaMemsetAsync(h->d_cost_tab.p, 0, (BVP_COST_BUCKETS + 1) * sizeof(float), h->stream));
        }
        if (!ensure_dev(h->d_inst_cost, size_t(n) * sizeof(float)))
            return fail(h, BVP_ERR_NOMEM, "cost record allocation failed");
        a.inst_cost = static_cast<float*>(h->d_inst_cost.p);
    }
    if (host_pts > 0) {
        bvp_status s = prepare_host_outputs(h, n, host_pts, a);
        if (s != BVP_OK) return s;
    }
    CU(cudaEventRecord(h->ev[0], h->stream));
    {
        long long np = (long long)n * h->desc.n_params;
        const double* src = d_params;
        void* dst = h->d_params_j.p;
        void* args[] = {&src, &dst, &np};
        const int blocks = int(std::min<long long>((np + 255) / 256 + 1, 4096));
        CU(cudaLaunchKernel((const void*)h->k_convert, dim3(blocks), dim3(256), args, 0, h->stream));
    }
    {
        int nn = n, ms = h->opt.max_subintervals;
        int cs = cap_scale(h);
        const int* ni = d_n_init;
        int* cap = static_cast<int*>(h->d_cap.p);
        bvp_i64* off = static_cast<bvp_i64*>(h->d_node_off.p);
        int* ord = static_cast<int*>(h->d_order.p);
        int* ctr = static_cast<int*>(h->d_counter.p);
        const float* tab = h->have_tab ? static_cast<const float*>(h->d_cost_tab.p) : nullptr;
        int gm = blk ? h->group_min : 0;
        void* args[] = {&nn, &ni, &ms, &cs, &cap, &off, &ord, &ctr, &tab, &gm};
        CU(cudaLaunchKernel((const void*)h->k_prep, dim3(1), dim3(1024), args, 0, h->stream));
    }
    if (wait_side) CU(cudaStreamWaitEvent(h->stream, h->ev_side, 0));   // the guesses on the grid
    // the launch-shape tuner times the warp-only kernels; a block-mode launch drops its pending sample
    int var = 0;
    if (blk) h->tune.pending = -1;
    else var = fused_variant(h, n, y0_mode);
    CU(cudaEventRecord(h->ev[1], h->stream));
    if (h->ho) CU(cudaMemsetAsync(a.pause_count, 0, 2 * sizeof(int), h->stream));
    a.deal_sms = std::max(1, h->sm_count);
    {
        void* args[] = {&a};
        const cudaKernel_t k = blk ? h->k_fused_blk : h->k_fused_v[var];
        const int occ = blk ? h->occ_blk : h->occ_v[var];
        CU(cudaLaunchKernel((const void*)k, dim3(resident_grid(h, n, occ)), dim3(128), args, 0, h->stream));
    }
    if (h->ho) {
        bvp_status s = ho_rounds(h, a, n);
        if (s != BVP_OK) return s;
    }
    CU(cudaEventRecord(h->ev[2], h->stream));
    if (learn) {
        int nn = n, blend = h->have_tab ? 1 : 0;
        const int* ni = d_n_init;
        const float* cost = a.inst_cost;
        float* tab = static_cast<float*>(h->d_cost_tab.p);
        void* args[] = {&nn, &ni, &cost, &tab, &blend};
        CU(cudaLaunchKernel((const void*)h->k_learn, dim3(1), dim3(1024), args, 0, h->stream));
        h->have_tab = true;
        --h->learn_left;
    }
    h->last_n = n;
    h->last_tot = tot;
    h->stages_ok = h->opt.want_stages != 0;
    return BVP_OK;
}

// host pointer of pinned memory as the device sees it (the same pointer under unified addressing)
static void* dev_view_raw(void* p) {
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, p, 0) != cudaSuccess) return nullptr;
    return d;
}
#define dev_view_d(p) static_cast<double*>(dev_view_raw(p))

static bvp_status grow_outputs(bvp_handle* h, long long pts) {
    const int M = h->L.M;
    const bool stages = h->opt.want_stages != 0;
    if (!ensure_host(h->h_mesh, size_t(pts) * 8) || !ensure_host(h->h_y, size_t(pts) * M * 8) ||
        (stages && (!ensure_host(h->h_K, size_t(pts) * h->L.S * M * 8) ||
                    !ensure_host(h->h_KI, size_t(pts) * h->L.NSXA * M * 8))))
        return fail(h, BVP_ERR_NOMEM, "output allocation failed");
    h->out_cap = pts;
    return BVP_OK;
}

static bvp_status launch_pack(bvp_handle* h, int n) {
    BvpArgs a;
    fill_args(h, a, n, h->last_tot, 0, static_cast<const double*>(h->d_params.p), nullptr, nullptr, nullptr, nullptr);
    const long long* oo = static_cast<const long long*>(h->d_out_off.p);
    long long cap = h->out_cap;
    double* om = dev_view_d(h->h_mesh.p);
    double* oy = dev_view_d(h->h_y.p);
    const bool stages = h->opt.want_stages != 0;
    int ws = stages ? 1 : 0;
    double* oK = stages ? dev_view_d(h->h_K.p) : nullptr;
    double* oKI = stages ? dev_view_d(h->h_KI.p) : nullptr;
    if (!om || !oy || (stages && (!oK || !oKI))) return fail(h, BVP_ERR_CUDA, "host output not mapped");
    void* args[] = {&a, &oo, &cap, &om, &oy, &ws, &oK, &oKI};
    const int blocks = (n * 32 + 255) / 256;
    CU(cudaLaunchKernel((const void*)h->k_pack, dim3(std::max(1, blocks)), dim3(256), args, 0, h->stream));
    return BVP_OK;
}

// Brings per-instance state and packed solutions of the last solve to the host: the offsets
// and the packing run on the device right behind the solve and write into pinned host memory
// the device maps (no separate copies, one synchronisation); a batch larger than the outputs
// hold grows them and packs once more.
static bvp_status finish(bvp_handle* h, bvp_results* out) {
    const int n = h->last_n;
    if (!ensure_host(h->h_st, size_t(n) * sizeof(BvpInstState)) || !ensure_host(h->h_off, size_t(n + 1) * 8) ||
        !ensure_dev(h->d_out_off, size_t(n + 1) * 8))
        return fail(h, BVP_ERR_NOMEM, "pinned allocation failed");
    if (h->out_cap == 0) {
        bvp_status s0 = grow_outputs(h, 1024);
        if (s0 != BVP_OK) return s0;
    }
    {
        int nn = n;
        const BvpInstState* dst_ = static_cast<const BvpInstState*>(h->d_st.p);
        long long* doff = static_cast<long long*>(h->d_out_off.p);
        long long* hoff = static_cast<long long*>(dev_view_raw(h->h_off.p));
        BvpInstState* hst = static_cast<BvpInstState*>(dev_view_raw(h->h_st.p));
        if (!hoff || !hst) return fail(h, BVP_ERR_CUDA, "host output not mapped");
        void* args[] = {&nn, &dst_, &doff, &hoff, &hst};
        CU(cudaLaunchKernel((const void*)h->k_offsets, dim3(1), dim3(1024), args, 0, h->stream));
    }
    bvp_status s = launch_pack(h, n);
    if (s != BVP_OK) return s;
    CU(cudaStreamSynchronize(h->stream));
    const int64_t* off = static_cast<const int64_t*>(h->h_off.p);
    const long long tot_out = off[n];
    if (tot_out > h->out_cap) {
        s = grow_outputs(h, tot_out + tot_out / 4);
        if (s != BVP_OK) return s;
        s = launch_pack(h, n);
        if (s != BVP_OK) return s;
        CU(cudaStreamSynchronize(h->stream));
    }
    float ms0 = 0, ms1 = 0;
    cudaEventElapsedTime(&ms0, h->ev[0], h->ev[2]);
    cudaEventElapsedTime(&ms1, h->ev[1], h->ev[2]);
    h->timing_ms[0] = ms0;
    h->timing_ms[1] = ms1;
    const BvpInstState* st = static_cast<const BvpInstState*>(h->h_st.p);
    h->st.assign(st, st + n);
    h->offsets.assign(off, off + n + 1);
    if (out) {
        for (int q = 0; q < n; ++q) {
            if (out->retcode) out->retcode[q] = st[q].retcode;
            if (out->n_nodes) out->n_nodes[q] = st[q].N;
            if (out->newton_iters) out->newton_iters[q] = st[q].newton_iters;
            if (out->rounds) out->rounds[q] = st[q].rounds;
            if (out->defect) out->defect[q] = st[q].defect;
            if (out->resid) out->resid[q] = st[q].resid;
            if (out->global_err) out->global_err[q] = st[q].global_err;
        }
    }
    h->have_results = true;
    h->pending_device = false;
    return BVP_OK;
}

// Host outputs for a solve whose kernel writes its results to pinned host memory as each
// instance finishes (the host calls: bvp_solve_batch, bvp_solve_batch_warm). pts_guess sizes
// the arrays on first use; later calls keep the largest size seen.
static bvp_status prepare_host_outputs(bvp_handle* h, int n, long long pts_guess, BvpArgs& a) {
    if (!ensure_host(h->h_st, size_t(n) * sizeof(BvpInstState)) || !ensure_host(h->h_off, size_t(n + 1) * 8) ||
        !ensure_dev(h->d_out_off, size_t(n + 1) * 8))
        return fail(h, BVP_ERR_NOMEM, "pinned allocation failed");
    if (h->out_cap < pts_guess) {
        bvp_status s = grow_outputs(h, pts_guess + pts_guess / 4);
        if (s != BVP_OK) return s;
    }
    const bool stages = h->opt.want_stages != 0;
    a.host_mesh = dev_view_d(h->h_mesh.p);
    a.host_y = dev_view_d(h->h_y.p);
    a.host_K = stages ? dev_view_d(h->h_K.p) : nullptr;
    a.host_KI = stages ? dev_view_d(h->h_KI.p) : nullptr;
    a.host_start = static_cast<bvp_i64*>(dev_view_raw(h->h_off.p));
    a.host_st = static_cast<BvpInstState*>(dev_view_raw(h->h_st.p));
    a.out_cursor = reinterpret_cast<unsigned long long*>(static_cast<char*>(h->d_counter.p) + 8);
    a.host_cap = h->out_cap;
    if (!a.host_mesh || !a.host_y || !a.host_start || !a.host_st || (stages && (!a.host_K || !a.host_KI)))
        return fail(h, BVP_ERR_CUDA, "host output not mapped");
    CU(cudaMemsetAsync(a.out_cursor, 0, 8, h->stream));
    return BVP_OK;
}

// Completes a solve launched with host outputs: one synchronisation; the offsets are the
// instances' starts (completion order) and offsets[n] the total. Instances that did not fit
// are packed again, in instance order, after the arrays grow.
static bvp_status finish_host(bvp_handle* h, bvp_results* out) {
    const int n = h->last_n;
    CU(cudaStreamSynchronize(h->stream));
    const BvpInstState* st = static_cast<const BvpInstState*>(h->h_st.p);
    int64_t* off = static_cast<int64_t*>(h->h_off.p);
    long long total = 0;
    bool overflow = false;
    for (int q = 0; q < n; ++q) {
        total += st[q].N;
        overflow |= off[q] < 0;
    }
    if (overflow) return finish(h, out);
    off[n] = total;
    float ms0 = 0, ms1 = 0;
    cudaEventElapsedTime(&ms0, h->ev[0], h->ev[2]);
    cudaEventElapsedTime(&ms1, h->ev[1], h->ev[2]);
    h->timing_ms[0] = ms0;
    h->timing_ms[1] = ms1;
    h->st.assign(st, st + n);
    h->offsets.assign(off, off + n + 1);
    if (out) {
        for (int q = 0; q < n; ++q) {
            if (out->retcode) out->retcode[q] = st[q].retcode;
            if (out->n_nodes) out->n_nodes[q] = st[q].N;
            if (out->newton_iters) out->newton_iters[q] = st[q].newton_iters;
            if (out->rounds) out->rounds[q] = st[q].rounds;
            if (out->defect) out->defect[q] = st[q].defect;
            if (out->resid) out->resid[q] = st[q].resid;
            if (out->global_err) out->global_err[q] = st[q].global_err;
        }
    }
    h->have_results = true;
    h->pending_device = false;
    return BVP_OK;
}

// ---- larger-state path (M > 8): the bl_* kernels, Newton and mesh rounds driven here --------
// The per-instance control flow is the one the fused kernel runs (solve_instance /
// newton_attempt with the FP64 residual throughout): Newton on ||F||_inf <= abstol with the
// stall and divergence tests, a backtracking retry from the same start, the defect, the
// mesh selection (sequential per instance: here), the transfer and the halving restart.
namespace {
struct LargeInst {
    int N = 0, cap = 0;
    long long off = 0;
    std::vector<double> mesh, h;
    int rounds = 0, retcode = BVP_RET_FAILURE, flags = 0, newton_total = 0;
    bool done = false;
    double defect = 0.0, resid = 0.0;
    // Newton attempt state
    int attempt = 0, iters = 0, why = 0, stall = 0, ls = 0, status = 0;  // status 0 running, 1 ok, 2 failed
    double nrm0 = 0, best = 0, f0 = 0, alpha = 1, sq = 0;
};
enum { LR_START = 0, LR_STEP = 1, LR_TRIAL = 2 };
double bits_to_double(unsigned long long b) {
    double v;
    std::memcpy(&v, &b, 8);
    return v;
}
}  // namespace

// bl_jacobian's dynamic shared memory: the staged parameters and 4 warps' workspaces
static size_t large_jac_smem(const bvp_handle* h) {
    const int P = h->desc.n_params;
    const size_t pb = P <= h->j_pmax ? (size_t(P) * size_t(h->js) + 15) / 16 * 16 : 0;
    return pb + 4 * h->j_warp_bytes;
}

static bvp_status large_run(bvp_handle* h, cudaKernel_t k, dim3 grid, dim3 block, size_t smem, BvpLargeArgs& a,
                            int* mode);

// Autotuner of the linear solve's block size (warps per instance = chunks of the mesh): on
// the first Newton step of the handle, every candidate from 3 warps up to the largest that
// fits is timed on the step's own systems (the solve reads the Jacobian blocks and the
// residual and writes only the step and its elimination records, so rerunning it is
// harmless), and the fastest is kept for the handle's life. Fewer warps per instance let
// more instances share an SM; more warps shorten each instance's chain of eliminations.
static bvp_status large_tune_linsolve(bvp_handle* h, BvpLargeArgs& a, int n_active) {
    const int wmax = h->l_threads / 32;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return fail(h, BVP_ERR_CUDA, "autotuner: event creation failed");
    }
    float best = 0.0f;
    int best_w = wmax;
    bvp_status s = BVP_OK;
    for (int rep = 0; rep < 2 && s == BVP_OK; ++rep) {   // the first pass warms up
        for (int w = 3; w <= wmax && s == BVP_OK; ++w) {
            const size_t smem = size_t(w) * h->l_warp_bytes + h->l_dense_bytes;
            float ms = 0.0f;
            if (cudaEventRecord(e0, h->stream) != cudaSuccess) { s = fail(h, BVP_ERR_CUDA, "autotuner: event"); break; }
            s = large_run(h, h->kl_solve, dim3(unsigned(n_active)), dim3(unsigned(32 * w)), smem, a, nullptr);
            if (s != BVP_OK) break;
            if (cudaEventRecord(e1, h->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                s = fail(h, BVP_ERR_CUDA, "autotuner: timing");
                break;
            }
            if (rep == 1 && (w == 3 || ms < best)) { best = ms; best_w = w; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != BVP_OK) return s;
    h->l_threads = 32 * best_w;
    h->l_smem = size_t(best_w) * h->l_warp_bytes + h->l_dense_bytes;
    h->l_tuned = true;
    return BVP_OK;
}

static bvp_status large_run(bvp_handle* h, cudaKernel_t k, dim3 grid, dim3 block, size_t smem, BvpLargeArgs& a,
                            int* mode = nullptr) {
    void* args1[] = {&a};
    void* args2[] = {&a, mode};
    CU(cudaLaunchKernel((const void*)k, grid, block, mode ? args2 : args1, smem, h->stream));
    return BVP_OK;
}

// uploads the active list and returns the grid rows
static bvp_status large_active(bvp_handle* h, BvpLargeArgs& a, const std::vector<int>& ids) {
    a.n_active = int(ids.size());
    if (ids.empty()) return BVP_OK;
    CU(cudaMemcpyAsync(h->d_active.p, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice, h->stream));
    return BVP_OK;
}

static bvp_status large_per_node(bvp_handle* h, BvpLargeArgs& a, cudaKernel_t k, int maxN, int mode = -1) {
    if (a.n_active == 0) return BVP_OK;
    const int M = h->L.M;
    dim3 grid(unsigned((maxN * M + 255) / 256), unsigned(a.n_active));
    return large_run(h, k, grid, dim3(256), 0, a, mode >= 0 ? &mode : nullptr);
}

static bvp_status solve_large(bvp_handle* h, int n, const double* params, const int32_t* n_intervals,
                              const double* tspans, int y0_mode, const double* y0, bvp_results* out) {
    const int M = h->L.M, P = h->desc.n_params;
    const bvp_options& o = h->opt;
    std::vector<LargeInst> I(n);
    long long tot = 0;
    for (int q = 0; q < n; ++q) {
        const int ni = n_intervals[q];
        if (ni < 1) return fail(h, BVP_ERR_INVALID, "n_intervals must be >= 1");
        if (!(tspans[2 * q + 1] > tspans[2 * q])) return fail(h, BVP_ERR_INVALID, "tspan must satisfy t0 < t1");
        I[q].cap = std::max(ni, o.max_subintervals) + 1;
        I[q].off = tot;
        tot += I[q].cap;
    }
    bvp_status s = ensure_arena(h, tot, n, 1);
    if (s != BVP_OK) return s;
    const int js = h->js;
    if (!ensure_dev(h->d_bcres, size_t(n) * M * 8) || !ensure_dev(h->d_G, size_t(n) * 2 * M * M * js) ||
        !ensure_dev(h->d_lnorm, size_t(n) * 8) || !ensure_dev(h->d_lsq, size_t(n) * 8) ||
        !ensure_dev(h->d_ldnorm, size_t(n) * 8) || !ensure_dev(h->d_lbad, size_t(n) * 4) ||
        !ensure_dev(h->d_active, size_t(n) * 4) || !ensure_dev(h->d_N, size_t(n) * 4) ||
        !ensure_dev(h->d_newN, size_t(n) * 4))
        return fail(h, BVP_ERR_NOMEM, "device allocation failed");
    // inputs, meshes, initial guesses
    std::vector<long long> offs(n);
    std::vector<int> Ns(n);
    if (P) CU(cudaMemcpyAsync(h->d_params.p, params, size_t(n) * P * 8, cudaMemcpyHostToDevice, h->stream));
    {
        long long np = (long long)n * P;
        const double* src = static_cast<const double*>(h->d_params.p);
        void* dst = h->d_params_j.p;
        void* args[] = {&src, &dst, &np};
        if (np) CU(cudaLaunchKernel((const void*)h->kl_convert, dim3(256), dim3(256), args, 0, h->stream));
    }
    // initial meshes, spacings and guesses packed instance after instance, uploaded at once and
    // scattered into the arena by bl_scatter
    std::vector<long long> poff(n + 1, 0);
    for (int q = 0; q < n; ++q) poff[q + 1] = poff[q] + n_intervals[q] + 1;
    std::vector<double> pm(size_t(poff[n])), ph(size_t(poff[n])), py(size_t(poff[n]) * M);
    long long yoff = 0;
    for (int q = 0; q < n; ++q) {
        LargeInst& L = I[q];
        const int ni = n_intervals[q];
        const double t0 = tspans[2 * q], t1 = tspans[2 * q + 1];
        const double hh = (t1 - t0) / ni;   // range(t0; stop = t1, length = n + 1) (Core/utils.jl:694-700)
        L.N = ni + 1;
        L.mesh.resize(ni + 1);
        L.h.resize(ni);
        for (int i = 0; i <= ni; ++i) L.mesh[i] = (i == ni) ? t1 : std::fma(double(i), hh, t0);
        for (int i = 0; i < ni; ++i) L.h[i] = L.mesh[i + 1] - L.mesh[i];
        double* yq = py.data() + size_t(poff[q]) * M;
        if (y0_mode == 0) {
            for (int i = 0; i < L.N; ++i)
                for (int m = 0; m < M; ++m) yq[size_t(i) * M + m] = y0[size_t(q) * M + m];
        } else {
            std::memcpy(yq, y0 + yoff * M, size_t(L.N) * M * 8);
            yoff += L.N;
        }
        std::memcpy(pm.data() + poff[q], L.mesh.data(), size_t(L.N) * 8);
        std::memcpy(ph.data() + poff[q], L.h.data(), size_t(L.N - 1) * 8);
        offs[q] = L.off;
        Ns[q] = L.N;
    }
    CU(cudaMemcpyAsync(h->d_node_off.p, offs.data(), size_t(n) * 8, cudaMemcpyHostToDevice, h->stream));
    BvpLargeArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n_inst = n;
    a.n_params = P;
    a.active = static_cast<const int*>(h->d_active.p);
    a.params = static_cast<const double*>(h->d_params.p);
    a.params_j = h->d_params_j.p;
    a.node_off = static_cast<const bvp_i64*>(h->d_node_off.p);
    a.N = static_cast<const int*>(h->d_N.p);
    a.mesh = static_cast<double*>(h->d_mesh.p);
    a.h = static_cast<double*>(h->d_h.p);
    a.y = static_cast<double*>(h->d_y.p);
    a.ybase = static_cast<double*>(h->d_ybase.p);
    a.ybak = static_cast<double*>(h->d_ybak.p);
    a.K = static_cast<double*>(h->d_K.p);
    a.KI = static_cast<double*>(h->d_KI.p);
    a.F = static_cast<double*>(h->d_F.p);
    a.err = static_cast<double*>(h->d_err.p);
    a.inc = static_cast<double*>(h->d_inc.p);
    a.iold = static_cast<int*>(h->d_iold.p);
    a.bcres = static_cast<double*>(h->d_bcres.p);
    a.yj = h->d_yj.p;
    a.Sb = h->d_Sb.p;
    a.Rb = h->d_Rb.p;
    a.G = h->d_G.p;
    a.rec = h->d_rec.p;
    a.delta = h->d_delta.p;
    a.norm = static_cast<unsigned long long*>(h->d_lnorm.p);
    a.sq = static_cast<double*>(h->d_lsq.p);
    a.dnorm = static_cast<unsigned long long*>(h->d_ldnorm.p);
    a.bad = static_cast<int*>(h->d_lbad.p);
    a.tot = tot;
    a.transfer_inplace = o.transfer_inplace;
    a.newN = static_cast<const int*>(h->d_newN.p);
    {
        // the packed inputs go through scratch arrays of the arena that the solve rewrites
        // before reading (ybase, inc, err), then into place
        double* dpy = static_cast<double*>(h->d_ybase.p);
        double* dpm = static_cast<double*>(h->d_inc.p);
        double* dph = dpm + poff[n];
        long long* dpo = static_cast<long long*>(h->d_err.p);
        CU(cudaMemcpyAsync(dpy, py.data(), py.size() * 8, cudaMemcpyHostToDevice, h->stream));
        CU(cudaMemcpyAsync(dpm, pm.data(), pm.size() * 8, cudaMemcpyHostToDevice, h->stream));
        CU(cudaMemcpyAsync(dph, ph.data(), ph.size() * 8, cudaMemcpyHostToDevice, h->stream));
        CU(cudaMemcpyAsync(dpo, poff.data(), poff.size() * 8, cudaMemcpyHostToDevice, h->stream));
        int mxN = 2;
        for (int q = 0; q < n; ++q) mxN = std::max(mxN, I[q].N);
        const double* cpy = dpy;
        const double* cpm = dpm;
        const double* cph = dph;
        const long long* cpo = dpo;
        void* args[] = {&a, &cpm, &cph, &cpy, &cpo};
        CU(cudaLaunchKernel((const void*)h->kl_scatter, dim3(unsigned(std::min(64, (mxN * M + 255) / 256)), unsigned(n)),
                            dim3(256), args, 0, h->stream));
    }
    CU(cudaEventRecord(h->ev[0], h->stream));
    CU(cudaEventRecord(h->ev[1], h->stream));
    std::vector<unsigned long long> nb(n);
    std::vector<double> sqv(n);
    std::vector<int> badv(n);
    auto upload_N = [&]() -> bvp_status {
        for (int q = 0; q < n; ++q) Ns[q] = I[q].N;
        CU(cudaMemcpyAsync(h->d_N.p, Ns.data(), size_t(n) * 4, cudaMemcpyHostToDevice, h->stream));
        return BVP_OK;
    };
    auto maxN_of = [&](const std::vector<int>& ids) {
        int mx = 2;
        for (int q : ids) mx = std::max(mx, I[q].N);
        return mx;
    };
    s = upload_N();
    if (s != BVP_OK) return s;
    for (int round = 0;; ++round) {
        std::vector<int> act;
        for (int q = 0; q < n; ++q)
            if (!I[q].done) act.push_back(q);
        if (act.empty()) break;
        // ---- Newton (newton / newton_attempt) ----
        for (int q : act) {
            LargeInst& L = I[q];
            ++L.rounds;
            L.attempt = 0; L.iters = 0; L.why = LR_START; L.status = 0; L.stall = 0;
        }
        s = large_active(h, a, act);
        if (s != BVP_OK) return s;
        s = large_per_node(h, a, h->kl_copy, maxN_of(act), 3);   // ybak = y
        if (s != BVP_OK) return s;
        while (true) {
            std::vector<int> run;
            for (int q : act)
                if (I[q].status == 0) run.push_back(q);
            if (run.empty()) break;
            // residual at every running instance's current iterate
            s = large_active(h, a, run);
            if (s != BVP_OK) return s;
            CU(cudaMemsetAsync(h->d_lnorm.p, 0, size_t(n) * 8, h->stream));
            CU(cudaMemsetAsync(h->d_lsq.p, 0, size_t(n) * 8, h->stream));
            {
                const int mx = maxN_of(run);
                s = large_run(h, h->kl_res, dim3(unsigned((mx + 127) / 128), unsigned(run.size())), dim3(128), 0, a);
                if (s != BVP_OK) return s;
            }
            CU(cudaMemcpyAsync(nb.data(), h->d_lnorm.p, size_t(n) * 8, cudaMemcpyDeviceToHost, h->stream));
            CU(cudaMemcpyAsync(sqv.data(), h->d_lsq.p, size_t(n) * 8, cudaMemcpyDeviceToHost, h->stream));
            CU(cudaStreamSynchronize(h->stream));
            std::vector<int> step, restart;
            std::map<double, std::vector<int>> trials;
            auto attempt_failed = [&](LargeInst& L, int q) {
                if (L.attempt == 0 && o.linesearch_fallback) {
                    L.attempt = 1; L.iters = 0; L.why = LR_START; L.stall = 0;
                    L.flags |= 1;
                    restart.push_back(q);
                } else {
                    L.status = 2;
                }
            };
            for (int q : run) {
                LargeInst& L = I[q];
                const double nrm = bits_to_double(nb[q]);
                const double f1 = sqv[q];
                if (L.why == LR_TRIAL) {
                    if (!(std::isfinite(nrm) && f1 <= (1.0 - 2e-4 * L.alpha) * L.f0)) {
                        L.alpha *= 0.5;
                        if (++L.ls >= 20) { L.resid = nrm; attempt_failed(L, q); continue; }
                        trials[L.alpha].push_back(q);
                        continue;
                    }
                    L.why = LR_STEP;
                }
                L.resid = nrm;
                L.sq = f1;
                bool need_step = false;
                if (L.why == LR_START) {
                    if (!std::isfinite(nrm)) { attempt_failed(L, q); continue; }
                    if (nrm <= o.abstol) { L.status = 1; continue; }
                    L.nrm0 = nrm; L.best = nrm; L.stall = 0;
                    need_step = true;
                } else {
                    if (!std::isfinite(nrm)) { attempt_failed(L, q); continue; }
                    if (nrm <= o.abstol) { L.status = 1; continue; }
                    if (nrm > o.divergence_factor * L.nrm0) { attempt_failed(L, q); continue; }
                    if (nrm < L.best) { L.best = nrm; L.stall = 0; }
                    else if (++L.stall >= o.stall_steps) { attempt_failed(L, q); continue; }
                    need_step = true;
                }
                if (need_step) {
                    if (L.iters >= o.max_newton) { attempt_failed(L, q); continue; }
                    step.push_back(q);
                }
            }
            // restarts of the line-search attempt from the saved start
            if (!restart.empty()) {
                s = large_active(h, a, restart);
                if (s != BVP_OK) return s;
                s = large_per_node(h, a, h->kl_copy, maxN_of(restart), 4);   // y = ybak
                if (s != BVP_OK) return s;
            }
            // the line search's shorter trials (same direction, y = ybase + alpha delta)
            for (auto& kv : trials) {
                s = large_active(h, a, kv.second);
                if (s != BVP_OK) return s;
                a.alpha = kv.first;
                s = large_per_node(h, a, h->kl_update, maxN_of(kv.second));
                a.alpha = 0.0;
                if (s != BVP_OK) return s;
            }
            if (step.empty()) continue;
            // Newton steps: Jacobian blocks, factorisation and solve
            s = large_active(h, a, step);
            if (s != BVP_OK) return s;
            {
                const int mx = maxN_of(step);
                const int runs = (mx - 1 + 7) / 8 + 1;   // runs of 8 intervals, plus the BC warp
                s = large_run(h, h->kl_jac, dim3(unsigned((runs + 3) / 4), unsigned(step.size())), dim3(128),
                              large_jac_smem(h), a);
                if (s != BVP_OK) return s;
                if (!h->l_tuned) {
                    s = large_tune_linsolve(h, a, int(step.size()));
                    if (s != BVP_OK) return s;
                }
                s = large_run(h, h->kl_solve, dim3(unsigned(step.size())), dim3(unsigned(h->l_threads)), h->l_smem, a);
                if (s != BVP_OK) return s;
            }
            CU(cudaMemcpyAsync(badv.data(), h->d_lbad.p, size_t(n) * 4, cudaMemcpyDeviceToHost, h->stream));
            CU(cudaStreamSynchronize(h->stream));
            std::vector<int> plain, ls;
            restart.clear();
            for (int q : step) {
                LargeInst& L = I[q];
                if (badv[q]) { attempt_failed(L, q); continue; }
                ++L.iters;
                ++L.newton_total;
                if (L.attempt == 0) { plain.push_back(q); L.why = LR_STEP; }
                else { ls.push_back(q); L.f0 = L.sq; L.alpha = 1.0; L.ls = 0; L.why = LR_TRIAL; }
            }
            if (!restart.empty()) {
                s = large_active(h, a, restart);
                if (s != BVP_OK) return s;
                s = large_per_node(h, a, h->kl_copy, maxN_of(restart), 4);
                if (s != BVP_OK) return s;
            }
            if (!plain.empty()) {
                s = large_active(h, a, plain);
                if (s != BVP_OK) return s;
                a.alpha = 0.0;
                s = large_per_node(h, a, h->kl_update, maxN_of(plain));
                if (s != BVP_OK) return s;
            }
            if (!ls.empty()) {
                s = large_active(h, a, ls);
                if (s != BVP_OK) return s;
                s = large_per_node(h, a, h->kl_copy, maxN_of(ls), 0);   // ybase = y
                if (s != BVP_OK) return s;
                a.alpha = 1.0;
                s = large_per_node(h, a, h->kl_update, maxN_of(ls));
                a.alpha = 0.0;
                if (s != BVP_OK) return s;
            }
        }
        // ---- defect of the converged instances ----
        std::vector<int> conv;
        for (int q : act)
            if (I[q].status == 1) conv.push_back(q);
        std::vector<double> dn(n, 0.0);
        if (o.adaptive && !conv.empty()) {
            s = large_active(h, a, conv);
            if (s != BVP_OK) return s;
            CU(cudaMemsetAsync(h->d_ldnorm.p, 0, size_t(n) * 8, h->stream));
            const int mx = maxN_of(conv);
            s = large_run(h, h->kl_defect, dim3(unsigned((mx + 127) / 128), unsigned(conv.size())), dim3(128), 0, a);
            if (s != BVP_OK) return s;
            CU(cudaMemcpyAsync(nb.data(), h->d_ldnorm.p, size_t(n) * 8, cudaMemcpyDeviceToHost, h->stream));
            CU(cudaStreamSynchronize(h->stream));
            for (int q : conv) dn[q] = bits_to_double(nb[q]);
        }
        // ---- outer-loop decisions (solve!, mirk.jl:286-388) ----
        std::vector<int> refine, halve;
        for (int q : act) {
            LargeInst& L = I[q];
            const bool nl_ok = L.status == 1;
            if (!o.adaptive) { L.retcode = nl_ok ? BVP_RET_SUCCESS : BVP_RET_FAILURE; L.done = true; continue; }
            double error_norm = 2 * o.abstol;
            bool ok = nl_ok;
            if (ok) {
                error_norm = dn[q];
                L.defect = error_norm;
                ok = !(error_norm > o.defect_threshold) && !std::isnan(error_norm);
            }
            if (ok && error_norm > o.abstol) {
                refine.push_back(q);   // continues unless the mesh selection fails (below)
                continue;
            }
            int info_ok = 1;
            if (!ok) {
                if (2L * (L.N - 1) > o.max_subintervals || 2 * (L.N - 1) + 1 > L.cap) {
                    info_ok = 0;
                    if (2 * (L.N - 1) + 1 > L.cap) L.flags |= 2;
                } else {
                    halve.push_back(q);
                }
            }
            if (!(info_ok && error_norm > o.abstol)) {
                L.retcode = info_ok ? BVP_RET_SUCCESS : BVP_RET_FAILURE;
                L.done = true;
            }
        }
        // mesh selection (adaptivity.jl:23-75, 250-304) for the refined instances
        std::vector<int> moved;
        std::vector<int> newNs(n, 0);
        for (int q : refine) {
            LargeInst& L = I[q];
            const int nI = L.N - 1;
            std::vector<double> e(nI);
            CU(cudaMemcpy(e.data(), static_cast<const double*>(h->d_err.p) + L.off, size_t(nI) * 8, cudaMemcpyDeviceToHost));
            const double ex = 1.0 / (o.order + 1);
            double r1 = -INFINITY, r2 = 0.0;
            for (int i = 0; i < nI; ++i) { e[i] = std::pow(e[i] / o.abstol, ex); r1 = std::max(r1, e[i]); }
            for (int i = 0; i < nI; ++i) r2 += e[i];
            const double r3 = r2 / (L.N - 1);
            long n_pred = (long)std::nearbyint(1.3 * r2 + 1);
            const double n_ = 0.1 * nI;
            if (std::fabs(double(n_pred - nI)) < n_) n_pred = (long)std::nearbyint(nI + n_);
            std::vector<double> nm, nh;
            bool ok = true;
            if (r1 <= 1.0 * r3) {
                if (2L * nI > o.max_subintervals || 2 * nI + 1 > L.cap) ok = false;
                else {
                    nm.assign(2 * nI + 1, 0.0); nh.assign(2 * nI, 0.0);
                    for (int i = 0; i <= nI; ++i) nm[2 * i] = L.mesh[i];
                    for (int i = 0; i < nI; ++i) {
                        nm[2 * i + 1] = (L.mesh[i + 1] + L.mesh[i]) / 2.0;
                        nh[2 * i] = L.h[i] / 2.0; nh[2 * i + 1] = L.h[i] / 2.0;
                    }
                }
            } else {
                const long lb = L.N / 2, ub = 4L * (L.N - 1);
                long Nsub = std::min(std::max(n_pred, lb), ub);
                if (Nsub > o.max_subintervals || Nsub + 1 > L.cap) ok = false;
                else {
                    for (int i = 0; i < nI; ++i) e[i] /= L.h[i];
                    double tot_int = 0.0;
                    for (int k = 0; k < nI; ++k) tot_int += e[k] * L.h[k];
                    const double zeta = tot_int / double(Nsub);
                    nm.assign(Nsub + 1, 0.0);
                    nm[0] = L.mesh[0];
                    double t = L.mesh[0], integral = 0.0;
                    int k = 0, i = 0;
                    long guard = 4L * (nI + Nsub) + 64;
                    while (k < nI && --guard > 0) {
                        const double next_piece = e[k] * (L.mesh[k + 1] - t);
                        const double int_next = integral + next_piece;
                        if (int_next > zeta) {
                            const double pt = (zeta - integral) / e[k] + t;
                            if (i + 1 < Nsub) nm[i + 1] = pt;
                            t = pt; ++i; integral = 0.0;
                        } else {
                            integral = int_next; t = L.mesh[k + 1]; ++k;
                        }
                    }
                    nm[Nsub] = L.mesh[nI];
                    nh.resize(Nsub);
                    for (int j = 0; j < Nsub; ++j) nh[j] = nm[j + 1] - nm[j];
                }
            }
            if (!ok) { L.retcode = BVP_RET_FAILURE; L.done = true; continue; }
            const int Nn = int(nm.size());
            CU(cudaMemcpy(static_cast<double*>(h->d_mesh.p) + tot + L.off, nm.data(), size_t(Nn) * 8, cudaMemcpyHostToDevice));
            CU(cudaMemcpy(static_cast<double*>(h->d_h.p) + tot + L.off, nh.data(), size_t(Nn - 1) * 8, cudaMemcpyHostToDevice));
            newNs[q] = Nn;
            moved.push_back(q);
            L.mesh.swap(nm);
            L.h.swap(nh);
        }
        if (!moved.empty()) {
            CU(cudaMemcpyAsync(h->d_newN.p, newNs.data(), size_t(n) * 4, cudaMemcpyHostToDevice, h->stream));
            s = large_active(h, a, moved);
            if (s != BVP_OK) return s;
            s = large_run(h, h->kl_transfer, dim3(unsigned((moved.size() * 32 + 127) / 128)), dim3(128), 0, a);
            if (s != BVP_OK) return s;
            CU(cudaStreamSynchronize(h->stream));
            for (int q : moved) I[q].N = newNs[q];
        }
        // halving restart with a zero guess
        for (int q : halve) {
            LargeInst& L = I[q];
            const int nI = L.N - 1;
            std::vector<double> nm(2 * nI + 1), nh(2 * nI);
            for (int i = 0; i <= nI; ++i) nm[2 * i] = L.mesh[i];
            for (int i = 0; i < nI; ++i) {
                nm[2 * i + 1] = (L.mesh[i + 1] + L.mesh[i]) / 2.0;
                nh[2 * i] = L.h[i] / 2.0; nh[2 * i + 1] = L.h[i] / 2.0;
            }
            L.mesh.swap(nm); L.h.swap(nh);
            L.N = 2 * nI + 1;
            CU(cudaMemcpy(static_cast<double*>(h->d_mesh.p) + L.off, L.mesh.data(), size_t(L.N) * 8, cudaMemcpyHostToDevice));
            CU(cudaMemcpy(static_cast<double*>(h->d_h.p) + L.off, L.h.data(), size_t(L.N - 1) * 8, cudaMemcpyHostToDevice));
            CU(cudaMemset(static_cast<double*>(h->d_y.p) + L.off * M, 0, size_t(L.N) * M * 8));
        }
        s = upload_N();
        if (s != BVP_OK) return s;
        for (int q : act) {
            LargeInst& L = I[q];
            if (!L.done && L.rounds >= o.max_rounds) { L.retcode = BVP_RET_MAXITERS; L.done = true; }
        }
    }
    const bool stages = o.want_stages != 0;
    if (stages) {
        // the interpolant's extra stages at every instance's final mesh and solution (the
        // stages K are the last residual's, at the accepted iterate): the defect pass over all
        // instances writes them
        std::vector<int> all(n);
        int mx = 2;
        for (int q = 0; q < n; ++q) { all[q] = q; mx = std::max(mx, I[q].N); }
        s = upload_N();
        if (s != BVP_OK) return s;
        s = large_active(h, a, all);
        if (s != BVP_OK) return s;
        CU(cudaMemsetAsync(h->d_ldnorm.p, 0, size_t(n) * 8, h->stream));
        s = large_run(h, h->kl_defect, dim3(unsigned((mx + 127) / 128), unsigned(n)), dim3(128), 0, a);
        if (s != BVP_OK) return s;
    }
    CU(cudaEventRecord(h->ev[2], h->stream));
    // results: per-instance state and the packed mesh and solution (and stages)
    long long total = 0;
    for (int q = 0; q < n; ++q) total += I[q].N;
    if (h->out_cap < total) {
        s = grow_outputs(h, total);
        if (s != BVP_OK) return s;
    }
    h->st.assign(n, BvpInstState{});
    h->offsets.assign(n + 1, 0);
    double* hm = static_cast<double*>(h->h_mesh.p);
    double* hy = static_cast<double*>(h->h_y.p);
    for (int q = 0; q < n; ++q) {
        const LargeInst& L = I[q];
        BvpInstState& st = h->st[q];
        st.N = L.N; st.cur = 0; st.retcode = L.retcode; st.newton_iters = L.newton_total; st.rounds = L.rounds;
        st.flags = L.flags; st.defect = L.defect; st.resid = L.resid; st.global_err = std::nan("");
        const long long o0 = h->offsets[q];
        std::memcpy(hm + o0, L.mesh.data(), size_t(L.N) * 8);
        CU(cudaMemcpyAsync(hy + o0 * M, static_cast<const double*>(h->d_y.p) + L.off * M, size_t(L.N) * M * 8,
                           cudaMemcpyDeviceToHost, h->stream));
        if (stages) {
            const int SM = h->L.S * M, XM = h->L.NSXA * M;
            CU(cudaMemcpyAsync(static_cast<double*>(h->h_K.p) + o0 * SM, static_cast<const double*>(h->d_K.p) + L.off * SM,
                               size_t(L.N - 1) * SM * 8, cudaMemcpyDeviceToHost, h->stream));
            CU(cudaMemcpyAsync(static_cast<double*>(h->h_KI.p) + o0 * XM, static_cast<const double*>(h->d_KI.p) + L.off * XM,
                               size_t(L.N - 1) * XM * 8, cudaMemcpyDeviceToHost, h->stream));
        }
        h->offsets[q + 1] = o0 + L.N;
    }
    CU(cudaStreamSynchronize(h->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev[0], h->ev[2]);
    h->timing_ms[0] = ms;
    h->timing_ms[1] = ms;
    h->last_n = n;
    h->stages_ok = stages;
    h->la = a;
    h->la.n_inst = n;
    h->have_results = true;
    h->pending_device = false;
    if (out) {
        for (int q = 0; q < n; ++q) {
            const BvpInstState& st = h->st[q];
            if (out->retcode) out->retcode[q] = st.retcode;
            if (out->n_nodes) out->n_nodes[q] = st.N;
            if (out->newton_iters) out->newton_iters[q] = st.newton_iters;
            if (out->rounds) out->rounds[q] = st.rounds;
            if (out->defect) out->defect[q] = st.defect;
            if (out->resid) out->resid[q] = st.resid;
            if (out->global_err) out->global_err[q] = st.global_err;
        }
    }
    return BVP_OK;
}

bvp_status bvp_solve_batch(bvp_handle* h, int32_t n, const double* params, const int32_t* n_intervals,
                           const double* tspans, int32_t y0_mode, const double* y0, bvp_results* out) {
    if (!h) return BVP_ERR_INVALID;
    if (n < 1 || !n_intervals || !tspans || !y0 || (h->desc.n_params > 0 && !params) ||
        (y0_mode != 0 && y0_mode != 1))
        return fail(h, BVP_ERR_INVALID, "invalid arguments");
    if (h->large) return solve_large(h, n, params, n_intervals, tspans, y0_mode, y0, out);
    const int M = h->L.M;
    long long tot = 0, y0_vals = 0, pts = 0;
    int max_init = 0;
    for (int q = 0; q < n; ++q) {
        const int ni = n_intervals[q];
        if (ni < 1) return fail(h, BVP_ERR_INVALID, "n_intervals must be >= 1");
        if (!(tspans[2 * q + 1] > tspans[2 * q])) return fail(h, BVP_ERR_INVALID, "tspan must satisfy t0 < t1");
        pts += ni + 1;
        tot += cap_nodes(h, ni);
        y0_vals += (y0_mode == 1) ? (long long)(ni + 1) * M : M;
        max_init = std::max(max_init, ni);
    }
    bvp_status s = ensure_arena(h, tot, n, y0_vals);
    if (s != BVP_OK) return s;
    const int P = h->desc.n_params;
    const size_t b_params = size_t(n) * P * 8, b_ni = size_t(n) * 4, b_ts = size_t(n) * 16,
                 b_y0 = size_t(y0_vals) * 8, b_off = size_t(n) * 8;
    if (!ensure_host(h->h_in, b_params + b_ni + b_ts + b_y0 + b_off + 64))
        return fail(h, BVP_ERR_NOMEM, "pinned allocation failed");
    char* hp = static_cast<char*>(h->h_in.p);
    // the staging copy is part of the host -> device path
    std::memcpy(hp, params, b_params);
    std::memcpy(hp + b_params, n_intervals, b_ni);
    std::memcpy(hp + b_params + b_ni, tspans, b_ts);
    std::memcpy(hp + b_params + b_ni + b_ts, y0, b_y0);
    int64_t* yoff = reinterpret_cast<int64_t*>(hp + b_params + b_ni + b_ts + b_y0);
    if (y0_mode == 1) {
        long long acc = 0;
        for (int q = 0; q < n; ++q) { yoff[q] = acc; acc += n_intervals[q] + 1; }
    }
    if (b_params) CU(cudaMemcpyAsync(h->d_params.p, hp, b_params, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_n_init.p, hp + b_params, b_ni, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_tspans.p, hp + b_params + b_ni, b_ts, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_y0.p, hp + b_params + b_ni + b_ts, b_y0, cudaMemcpyHostToDevice, h->stream));
    if (y0_mode == 1) CU(cudaMemcpyAsync(h->d_y0_off.p, yoff, b_off, cudaMemcpyHostToDevice, h->stream));
    s = launch_solve(h, n, tot, y0_mode, static_cast<const double*>(h->d_params.p),
                     static_cast<const int*>(h->d_n_init.p), static_cast<const double*>(h->d_tspans.p),
                     static_cast<const double*>(h->d_y0.p), static_cast<const long long*>(h->d_y0_off.p), max_init,
                     nullptr, 0, pts);
    if (s != BVP_OK) return s;
    return finish_host(h, out);
}

// The surrogate's forward into the handle's grid buffer on the side stream, once the work
// enqueued so far on the handle's stream (the inputs' copies) is done; ev_side marks its end.
static bvp_status side_forward(bvp_handle* h, bvp_mlp* net, int n, const float* d_features) {
    CU(cudaEventRecord(h->ev_in, h->stream));
    CU(cudaStreamWaitEvent(h->side, h->ev_in, 0));
    if (bvp_mlp_forward_device(net, n, d_features, static_cast<float*>(h->d_grid.p), h->side) != BVP_OK)
        return fail(h, BVP_ERR_CUDA, "surrogate forward failed");
    CU(cudaEventRecord(h->ev_side, h->side));
    return BVP_OK;
}

bvp_status bvp_solve_batch_device_warm(bvp_handle* h, bvp_mlp* net, int32_t n, const float* d_features,
                                       int32_t n_grid, const double* d_params, const int32_t* d_n_intervals,
                                       const double* d_tspans, int32_t max_intervals) {
    if (!h) return BVP_ERR_INVALID;
    if (h->large) return fail(h, BVP_ERR_INVALID, "state dimension above 8: bvp_solve_batch and bvp_solve_batch_device only");
    if (!net || n < 1 || !d_features || n_grid < 2 || !d_n_intervals || !d_tspans || max_intervals < 1 ||
        (h->desc.n_params > 0 && !d_params))
        return fail(h, BVP_ERR_INVALID, "invalid arguments");
    const long long tot = (long long)n * cap_nodes(h, max_intervals);
    bvp_status s = ensure_arena(h, tot, n, 1);
    if (s != BVP_OK) return s;
    if (!ensure_dev(h->d_grid, size_t(n) * n_grid * h->L.M * 4)) return fail(h, BVP_ERR_NOMEM, "device allocation failed");
    s = side_forward(h, net, n, d_features);
    if (s != BVP_OK) return s;
    s = launch_solve(h, n, tot, 2, d_params, d_n_intervals, d_tspans, static_cast<const double*>(h->d_y0.p),
                     static_cast<const long long*>(h->d_y0_off.p), max_intervals,
                     static_cast<const float*>(h->d_grid.p), n_grid, 0, true);
    if (s != BVP_OK) return s;
    h->pending_device = true;
    h->have_results = false;
    return BVP_OK;
}

bvp_status bvp_solve_batch_warm(bvp_handle* h, bvp_mlp* net, int32_t n, int32_t n_features, const float* features,
                                int32_t n_grid, const double* params, const int32_t* n_intervals,
                                const double* tspans, const double* y0_plain, bvp_results* out,
                                int32_t* n_fallback) {
    if (!h) return BVP_ERR_INVALID;
    if (h->large) return fail(h, BVP_ERR_INVALID, "state dimension above 8: bvp_solve_batch and bvp_solve_batch_device only");
    const int M = h->L.M;
    if (!net || n < 1 || n_features < 1 || !features || n_grid < 2 || !n_intervals || !tspans || !y0_plain ||
        (h->desc.n_params > 0 && !params))
        return fail(h, BVP_ERR_INVALID, "invalid arguments");
    long long tot = 0, y0_vals = 0, pts = 0;
    int max_init = 0;
    for (int q = 0; q < n; ++q) {
        const int ni = n_intervals[q];
        if (ni < 1) return fail(h, BVP_ERR_INVALID, "n_intervals must be >= 1");
        if (!(tspans[2 * q + 1] > tspans[2 * q])) return fail(h, BVP_ERR_INVALID, "tspan must satisfy t0 < t1");
        pts += ni + 1;
        tot += cap_nodes(h, ni);
        y0_vals += (long long)(ni + 1) * M;
        max_init = std::max(max_init, ni);
    }
    (void)y0_vals;
    bvp_status s = ensure_arena(h, tot, n, 1);
    if (s != BVP_OK) return s;
    // inputs staged through pinned memory: parameters, tspans, interval counts, features
    const int P = h->desc.n_params;
    const int nfeat = n_features;
    const size_t b_params = size_t(n) * P * 8, b_ts = size_t(n) * 16, b_ni = size_t(n) * 4,
                 b_feat = size_t(n) * nfeat * 4;
    if (!ensure_host(h->h_in, b_params + b_ts + b_ni + b_feat + 64)) return fail(h, BVP_ERR_NOMEM, "pinned allocation failed");
    if (!ensure_dev(h->d_feat, b_feat) || !ensure_dev(h->d_grid, size_t(n) * n_grid * M * 4))
        return fail(h, BVP_ERR_NOMEM, "device allocation failed");
    char* hp = static_cast<char*>(h->h_in.p);
    std::memcpy(hp, params, b_params);
    std::memcpy(hp + b_params, tspans, b_ts);
    std::memcpy(hp + b_params + b_ts, n_intervals, b_ni);
    std::memcpy(hp + b_params + b_ts + b_ni, features, b_feat);
    if (b_params) CU(cudaMemcpyAsync(h->d_params.p, hp, b_params, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_tspans.p, hp + b_params, b_ts, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_n_init.p, hp + b_params + b_ts, b_ni, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_feat.p, hp + b_params + b_ts + b_ni, b_feat, cudaMemcpyHostToDevice, h->stream));
    s = side_forward(h, net, n, static_cast<const float*>(h->d_feat.p));
    if (s != BVP_OK) return s;
    // the solve resamples the grid guesses onto the initial meshes itself (y0_mode 2)
    s = launch_solve(h, n, tot, 2, static_cast<const double*>(h->d_params.p), static_cast<const int*>(h->d_n_init.p),
                     static_cast<const double*>(h->d_tspans.p), static_cast<const double*>(h->d_y0.p),
                     static_cast<const long long*>(h->d_y0_off.p), max_init, static_cast<const float*>(h->d_grid.p),
                     n_grid, pts, true);
    if (s != BVP_OK) return s;
    s = finish_host(h, nullptr);
    if (s != BVP_OK) return s;
    // plain-guess fallback for the instances the warm start did not bring to convergence
    std::vector<int> bad;
    for (int q = 0; q < n; ++q)
        if (h->st[q].retcode != BVP_RET_SUCCESS) bad.push_back(q);
    if (n_fallback) *n_fallback = int(bad.size());
    if (!bad.empty()) {
        std::vector<BvpInstState> st0 = h->st;
        std::vector<int64_t> off0 = h->offsets;
        const long long tot0 = off0[n];
        std::vector<double> mesh0(static_cast<const double*>(h->h_mesh.p), static_cast<const double*>(h->h_mesh.p) + tot0);
        std::vector<double> y00(static_cast<const double*>(h->h_y.p), static_cast<const double*>(h->h_y.p) + tot0 * M);
        const int nb = int(bad.size());
        std::vector<double> bp(size_t(nb) * P), bts(size_t(nb) * 2), by0(size_t(nb) * M);
        std::vector<int32_t> bni(nb);
        for (int k = 0; k < nb; ++k) {
            const int q = bad[k];
            for (int c = 0; c < P; ++c) bp[size_t(k) * P + c] = params[size_t(q) * P + c];
            bts[2 * k] = tspans[2 * q]; bts[2 * k + 1] = tspans[2 * q + 1];
            for (int m = 0; m < M; ++m) by0[size_t(k) * M + m] = y0_plain[size_t(q) * M + m];
            bni[k] = n_intervals[q];
        }
        s = bvp_solve_batch(h, nb, bp.data(), bni.data(), bts.data(), 0, by0.data(), nullptr);
        if (s != BVP_OK) return s;
        std::vector<BvpInstState> st1 = h->st;
        std::vector<int64_t> off1 = h->offsets;
        std::vector<double> mesh1(static_cast<const double*>(h->h_mesh.p), static_cast<const double*>(h->h_mesh.p) + off1[nb]);
        std::vector<double> y1(static_cast<const double*>(h->h_y.p), static_cast<const double*>(h->h_y.p) + off1[nb] * M);
        std::vector<int> slot(n, -1);
        for (int k = 0; k < nb; ++k) slot[bad[k]] = k;
        h->st.resize(n);
        h->offsets.assign(n + 1, 0);
        for (int q = 0; q < n; ++q) {
            h->st[q] = slot[q] >= 0 ? st1[slot[q]] : st0[q];
            h->offsets[q + 1] = h->offsets[q] + h->st[q].N;
        }
        const long long totm = h->offsets[n];
        if (!ensure_host(h->h_mesh, size_t(totm) * 8) || !ensure_host(h->h_y, size_t(totm) * M * 8))
            return fail(h, BVP_ERR_NOMEM, "pinned allocation failed");
        double* hm = static_cast<double*>(h->h_mesh.p);
        double* hy = static_cast<double*>(h->h_y.p);
        for (int q = 0; q < n; ++q) {
            const int k = slot[q];
            const double* sm = k >= 0 ? &mesh1[off1[k]] : &mesh0[off0[q]];
            const double* sy = k >= 0 ? &y1[off1[k] * M] : &y00[off0[q] * M];
            std::memcpy(hm + h->offsets[q], sm, size_t(h->st[q].N) * 8);
            std::memcpy(hy + h->offsets[q] * M, sy, size_t(h->st[q].N) * M * 8);
        }
        h->last_n = n;
        h->stages_ok = false;  // the stages on the device belong to the fallback subset only
    }
    if (out) {
        for (int q = 0; q < n; ++q) {
            const BvpInstState& st = h->st[q];
            if (out->retcode) out->retcode[q] = st.retcode;
            if (out->n_nodes) out->n_nodes[q] = st.N;
            if (out->newton_iters) out->newton_iters[q] = st.newton_iters;
            if (out->rounds) out->rounds[q] = st.rounds;
            if (out->defect) out->defect[q] = st.defect;
            if (out->resid) out->resid[q] = st.resid;
            if (out->global_err) out->global_err[q] = st.global_err;
        }
    }
    return BVP_OK;
}

// The larger-state path (M > 8) drives its Newton steps from the host, so a solve on device
// inputs reads them back (on the handle's stream) and runs the host-buffer solve; it returns
// with the results in the handle, which bvp_fetch_results then reads.
static bvp_status solve_large_from_device(bvp_handle* h, int n, const double* d_params, const int32_t* d_n_intervals,
                                          const double* d_tspans, int y0_mode, const double* d_y0,
                                          const int64_t* d_y0_off, int max_intervals) {
    const int M = h->L.M, P = h->desc.n_params;
    if (n < 1 || !d_n_intervals || !d_tspans || !d_y0 || max_intervals < 1 || (y0_mode != 0 && y0_mode != 1) ||
        (y0_mode == 1 && !d_y0_off) || (P > 0 && !d_params))
        return fail(h, BVP_ERR_INVALID, "invalid arguments");
    std::vector<int32_t> ni(n);
    std::vector<double> ts(size_t(n) * 2), pr(size_t(n) * std::max(P, 1));
    CU(cudaMemcpyAsync(ni.data(), d_n_intervals, size_t(n) * 4, cudaMemcpyDeviceToHost, h->stream));
    CU(cudaMemcpyAsync(ts.data(), d_tspans, size_t(n) * 16, cudaMemcpyDeviceToHost, h->stream));
    if (P > 0) CU(cudaMemcpyAsync(pr.data(), d_params, size_t(n) * P * 8, cudaMemcpyDeviceToHost, h->stream));
    std::vector<int64_t> off;
    if (y0_mode == 1) {
        off.resize(n);
        CU(cudaMemcpyAsync(off.data(), d_y0_off, size_t(n) * 8, cudaMemcpyDeviceToHost, h->stream));
    }
    CU(cudaStreamSynchronize(h->stream));
    for (int q = 0; q < n; ++q)
        if (ni[q] < 1 || ni[q] > max_intervals) return fail(h, BVP_ERR_INVALID, "n_intervals outside 1..max_intervals");
    std::vector<double> y0;
    if (y0_mode == 0) {
        y0.resize(size_t(n) * M);
        CU(cudaMemcpyAsync(y0.data(), d_y0, y0.size() * 8, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaStreamSynchronize(h->stream));
    } else {
        // the per-instance blocks of the device array, packed in instance order
        long long need = 0, packed = 0;
        for (int q = 0; q < n; ++q) {
            if (off[q] < 0) return fail(h, BVP_ERR_INVALID, "negative y0 offset");
            need = std::max<long long>(need, off[q] + ni[q] + 1);
            packed += ni[q] + 1;
        }
        std::vector<double> all(size_t(need) * M);
        CU(cudaMemcpyAsync(all.data(), d_y0, all.size() * 8, cudaMemcpyDeviceToHost, h->stream));
        CU(cudaStreamSynchronize(h->stream));
        y0.reserve(size_t(packed) * M);
        for (int q = 0; q < n; ++q)
            y0.insert(y0.end(), all.begin() + off[q] * M, all.begin() + (off[q] + ni[q] + 1) * M);
    }
    return solve_large(h, n, P > 0 ? pr.data() : nullptr, ni.data(), ts.data(), y0_mode, y0.data(), nullptr);
}

bvp_status bvp_solve_batch_device(bvp_handle* h, int32_t n, const double* d_params, const int32_t* d_n_intervals,
                                  const double* d_tspans, int32_t y0_mode, const double* d_y0,
                                  const int64_t* d_y0_off, int32_t max_intervals) {
    if (!h) return BVP_ERR_INVALID;
    if (h->large)
        return solve_large_from_device(h, n, d_params, d_n_intervals, d_tspans, y0_mode, d_y0, d_y0_off, max_intervals);
    if (n < 1 || !d_n_intervals || !d_tspans || !d_y0 || max_intervals < 1 || (y0_mode == 1 && !d_y0_off))
        return fail(h, BVP_ERR_INVALID, "invalid arguments");
    const long long tot = (long long)n * cap_nodes(h, max_intervals);
    bvp_status s = ensure_arena(h, tot, n, 1);
    if (s != BVP_OK) return s;
    const double* dp = d_params ? d_params : static_cast<const double*>(h->d_params.p);
    s = launch_solve(h, n, tot, y0_mode, dp, d_n_intervals, d_tspans, d_y0,
                     reinterpret_cast<const long long*>(d_y0_off), max_intervals);
    if (s != BVP_OK) return s;
    h->pending_device = true;
    h->have_results = false;
    return BVP_OK;
}

bvp_status bvp_solve_batch_device_grid(bvp_handle* h, int32_t n, const double* d_params,
                                       const int32_t* d_n_intervals, const double* d_tspans, const float* d_grid,
                                       int32_t n_grid, int32_t max_intervals) {
    if (!h) return BVP_ERR_INVALID;
    if (h->large) return fail(h, BVP_ERR_INVALID, "state dimension above 8: bvp_solve_batch and bvp_solve_batch_device only");
    if (n < 1 || !d_n_intervals || !d_tspans || !d_grid || n_grid < 2 || max_intervals < 1 ||
        (h->desc.n_params > 0 && !d_params))
        return fail(h, BVP_ERR_INVALID, "invalid arguments");
    const long long tot = (long long)n * cap_nodes(h, max_intervals);
    bvp_status s = ensure_arena(h, tot, n, 1);
    if (s != BVP_OK) return s;
    s = launch_solve(h, n, tot, 2, d_params, d_n_intervals, d_tspans, static_cast<const double*>(h->d_y0.p),
                     static_cast<const long long*>(h->d_y0_off.p), max_intervals, d_grid, n_grid);
    if (s != BVP_OK) return s;
    h->pending_device = true;
    h->have_results = false;
    return BVP_OK;
}

bvp_status bvp_fetch_results(bvp_handle* h, bvp_results* out) {
    if (!h) return BVP_ERR_INVALID;
    if (!h->pending_device && !h->have_results) return fail(h, BVP_ERR_STATE, "no solve to fetch");
    if (h->have_results && !h->pending_device) {
        if (out) {
            for (int q = 0; q < h->last_n; ++q) {
                const BvpInstState& st = h->st[q];
                if (out->retcode) out->retcode[q] = st.retcode;
                if (out->n_nodes) out->n_nodes[q] = st.N;
                if (out->newton_iters) out->newton_iters[q] = st.newton_iters;
                if (out->rounds) out->rounds[q] = st.rounds;
                if (out->defect) out->defect[q] = st.defect;
                if (out->resid) out->resid[q] = st.resid;
                if (out->global_err) out->global_err[q] = st.global_err;
            }
        }
        return BVP_OK;
    }
    return finish(h, out);
}

bvp_status bvp_dense_output(bvp_handle* h, int32_t nq, const double* tq, int32_t deriv, double* out) {
    if (!h) return BVP_ERR_INVALID;
    if (!h->have_results && !h->pending_device) return fail(h, BVP_ERR_STATE, "no solve to interpolate");
    if (!h->stages_ok) return fail(h, BVP_ERR_STATE, "dense output needs want_stages = 1 and a solve without fallback");
    if (nq < 1 || !tq || !out) return fail(h, BVP_ERR_INVALID, "invalid arguments");
    const int n = h->last_n, M = h->L.M;
    DevBuf dt, dout;
    bvp_status s = BVP_OK;
    do {
        if (!ensure_dev(dt, size_t(n) * nq * 8) || !ensure_dev(dout, size_t(n) * nq * M * 8)) {
            s = fail(h, BVP_ERR_NOMEM, "device allocation failed");
            break;
        }
        if (cudaMemcpyAsync(dt.p, tq, size_t(n) * nq * 8, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) { s = fail(h, BVP_ERR_CUDA, "H2D"); break; }
        int nqq = nq, dv = deriv;
        const double* tp = static_cast<const double*>(dt.p);
        double* op = static_cast<double*>(dout.p);
        cudaError_t e;
        if (h->large) {
            // the larger-state kernels keep the final point counts in d_N (uploaded by the solve)
            void* args[] = {&h->la, &nqq, &tp, &dv, &op};
            e = cudaLaunchKernel((const void*)h->kl_dense, dim3((n * 32 + 127) / 128), dim3(128), args, 0, h->stream);
        } else {
            BvpArgs a;
            fill_args(h, a, n, h->last_tot, 0, static_cast<const double*>(h->d_params.p), nullptr, nullptr, nullptr, nullptr);
            void* args[] = {&a, &nqq, &tp, &dv, &op};
            e = cudaLaunchKernel((const void*)h->k_dense, dim3((n * 32 + 127) / 128), dim3(128), args, 0, h->stream);
        }
        if (e != cudaSuccess) { s = fail(h, BVP_ERR_CUDA, "dense launch"); break; }
        if (cudaMemcpyAsync(out, dout.p, size_t(n) * nq * M * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) { s = fail(h, BVP_ERR_CUDA, "D2H"); break; }
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) { s = fail(h, BVP_ERR_CUDA, "sync"); break; }
    } while (0);
    if (dt.p) cudaFree(dt.p);
    if (dout.p) cudaFree(dout.p);
    return s;
}

bvp_status bvp_get_tuning(bvp_handle* h, int32_t* threads) {
    if (!h || !threads) return BVP_ERR_INVALID;
    threads[0] = (h->large && h->l_tuned) ? h->l_threads : 0;
    return BVP_OK;
}

bvp_status bvp_get_fused_tuning(bvp_handle* h, int32_t* blocks_per_sm, int32_t* tuned, float* ms) {
    if (!h || !blocks_per_sm) return BVP_ERR_INVALID;
    *blocks_per_sm = h->large ? 0 : kFusedBlocks[h->fused_pick];
    if (tuned) *tuned = h->tune.done ? 1 : 0;
    if (ms)
        for (int c = 0; c < 3; ++c) ms[c] = h->tune.cnt[c] > 0 ? h->tune.sum[c] / h->tune.cnt[c] : 0.0f;
    return BVP_OK;
}

bvp_status bvp_get_block_mode(bvp_handle* h, int32_t* block_min, int32_t* last) {
    if (!h || !block_min) return BVP_ERR_INVALID;
    *block_min = h->group_min;
    if (last) *last = h->last_blk ? 1 : 0;
    return BVP_OK;
}

bvp_status bvp_get_work_order(bvp_handle* h, int32_t* learned, float* costs, int32_t n_costs) {
    if (!h || !learned) return BVP_ERR_INVALID;
    *learned = h->have_tab ? 1 : 0;
    if (costs && n_costs > 0) {
        const int k = std::min(n_costs, BVP_COST_BUCKETS + 1);
        if (!h->have_tab) {
            std::fill(costs, costs + k, 0.0f);
        } else {
            CU(cudaMemcpyAsync(costs, h->d_cost_tab.p, size_t(k) * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
            CU(cudaStreamSynchronize(h->stream));
        }
    }
    return BVP_OK;
}

bvp_status bvp_last_timing(bvp_handle* h, double* ms2) {
    if (!h || !ms2) return BVP_ERR_INVALID;
    if (h->pending_device) {
        CU(cudaStreamSynchronize(h->stream));
        float ms0 = 0, ms1 = 0;
        cudaEventElapsedTime(&ms0, h->ev[0], h->ev[2]);
        cudaEventElapsedTime(&ms1, h->ev[1], h->ev[2]);
        h->timing_ms[0] = ms0;
        h->timing_ms[1] = ms1;
    }
    ms2[0] = h->timing_ms[0];
    ms2[1] = h->timing_ms[1];
    return BVP_OK;
}

bvp_status bvp_get_solution(bvp_handle* h, int32_t inst, double* mesh, double* y, int32_t cap, int32_t* n_nodes) {
    if (!h) return BVP_ERR_INVALID;
    if (!h->have_results) return fail(h, BVP_ERR_STATE, "no results");
    if (inst < 0 || inst >= h->last_n) return fail(h, BVP_ERR_INVALID, "instance out of range");
    const int64_t o = h->offsets[inst];
    const int N = h->st[inst].N;
    if (n_nodes) *n_nodes = N;
    if (cap < N) return fail(h, BVP_ERR_INVALID, "capacity too small");
    const int M = h->L.M;
    if (mesh) std::memcpy(mesh, static_cast<const double*>(h->h_mesh.p) + o, size_t(N) * 8);
    if (y) std::memcpy(y, static_cast<const double*>(h->h_y.p) + o * M, size_t(N) * M * 8);
    return BVP_OK;
}

bvp_status bvp_get_packed(bvp_handle* h, const int64_t** offsets, const double** mesh, const double** y,
                          const double** K, const double** KI) {
    if (!h) return BVP_ERR_INVALID;
    if (!h->have_results) return fail(h, BVP_ERR_STATE, "no results");
    if (offsets) *offsets = h->offsets.data();
    if (mesh) *mesh = static_cast<const double*>(h->h_mesh.p);
    if (y) *y = static_cast<const double*>(h->h_y.p);
    if (K) *K = h->stages_ok ? static_cast<const double*>(h->h_K.p) : nullptr;
    if (KI) *KI = h->stages_ok ? static_cast<const double*>(h->h_KI.p) : nullptr;
    return BVP_OK;
}

bvp_status bvp_eval_stage(bvp_handle* h, int32_t stage, int32_t n, const double* params, const int32_t* n_nodes,
                          const double* mesh, const double* y, double* norm, double* F, double* bc_res,
                          double* K, double* S, double* R, double* delta, double* err) {
    if (!h) return BVP_ERR_INVALID;
    if (h->large) return fail(h, BVP_ERR_INVALID, "state dimension above 8: bvp_solve_batch and bvp_solve_batch_device only");
    if (h->firk) return fail(h, BVP_ERR_INVALID, "the stage kernels are MIRK's: not available on the FIRK path");
    if (stage < 0 || stage > 3 || n < 1 || !n_nodes || !mesh || !y || (h->desc.n_params > 0 && !params))
        return fail(h, BVP_ERR_INVALID, "invalid arguments");
    const BvpLayout& L = h->L;
    const int M = L.M, P = h->desc.n_params, js = h->js;
    std::vector<long long> off(n + 1, 0);
    std::vector<int> cap(n), order(n);
    for (int q = 0; q < n; ++q) {
        if (n_nodes[q] < 2) return fail(h, BVP_ERR_INVALID, "n_nodes must be >= 2");
        cap[q] = n_nodes[q];
        off[q + 1] = off[q] + n_nodes[q];
        order[q] = q;
    }
    const long long tot = off[n];
    bvp_status s = ensure_arena(h, tot, n, 1);
    if (s != BVP_OK) return s;
    std::vector<double> hh(size_t(tot), 0.0);
    std::vector<BvpInstState> st(n);
    for (int q = 0; q < n; ++q) {
        for (int i = 0; i + 1 < n_nodes[q]; ++i) hh[off[q] + i] = mesh[off[q] + i + 1] - mesh[off[q] + i];
        std::memset(&st[q], 0, sizeof(BvpInstState));
        st[q].N = n_nodes[q];
    }
    CU(cudaMemcpyAsync(h->d_mesh.p, mesh, size_t(tot) * 8, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_h.p, hh.data(), size_t(tot) * 8, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_y.p, y, size_t(tot) * M * 8, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_node_off.p, off.data(), size_t(n) * 8, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_cap.p, cap.data(), size_t(n) * 4, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_order.p, order.data(), size_t(n) * 4, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(h->d_st.p, st.data(), size_t(n) * sizeof(BvpInstState), cudaMemcpyHostToDevice, h->stream));
    if (P > 0) CU(cudaMemcpyAsync(h->d_params.p, params, size_t(n) * P * 8, cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemsetAsync(h->d_counter.p, 0, 16, h->stream));
    {
        long long np = (long long)n * P;
        const double* src = static_cast<const double*>(h->d_params.p);
        void* dst = h->d_params_j.p;
        void* args[] = {&src, &dst, &np};
        CU(cudaLaunchKernel((const void*)h->k_convert, dim3(64), dim3(256), args, 0, h->stream));
    }
    BvpArgs a;
    fill_args(h, a, n, tot, 0, static_cast<const double*>(h->d_params.p), nullptr, nullptr, nullptr, nullptr);
    double* dn = static_cast<double*>(h->d_norm.p);
    int stg = stage;
    void* args[] = {&a, &stg, &dn};
    CU(cudaLaunchKernel((const void*)h->k_stage, dim3(fused_grid(h, n)), dim3(128), args, 0, h->stream));
    CU(cudaStreamSynchronize(h->stream));
    if (norm) CU(cudaMemcpy(norm, dn, size_t(n) * 8, cudaMemcpyDeviceToHost));
    if (F) CU(cudaMemcpy(F, h->d_F.p, size_t(tot) * M * 8, cudaMemcpyDeviceToHost));
    if (K) CU(cudaMemcpy(K, h->d_K.p, size_t(tot) * L.S * M * 8, cudaMemcpyDeviceToHost));
    if (err) CU(cudaMemcpy(err, h->d_err.p, size_t(tot) * 8, cudaMemcpyDeviceToHost));
    if (bc_res) {
        std::vector<double> scr(size_t(n) * L.SCRW);
        CU(cudaMemcpy(scr.data(), h->d_scr.p, scr.size() * 8, cudaMemcpyDeviceToHost));
        for (int q = 0; q < n; ++q)
            for (int m = 0; m < M; ++m) bc_res[q * M + m] = scr[size_t(q) * L.SCRW + L.SCR_BCRES + m];
    }
    auto fetch_jt = [&](const DevBuf& b, double* dst, size_t count) -> bvp_status {
        if (js == 8) {
            CU(cudaMemcpy(dst, b.p, count * 8, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> tmp(count);
            CU(cudaMemcpy(tmp.data(), b.p, count * 4, cudaMemcpyDeviceToHost));
            for (size_t k = 0; k < count; ++k) dst[k] = tmp[k];
        }
        return BVP_OK;
    };
    if (S && (s = fetch_jt(h->d_Sb, S, size_t(tot) * M * M)) != BVP_OK) return s;
    if (R && (s = fetch_jt(h->d_Rb, R, size_t(tot) * M * M)) != BVP_OK) return s;
    if (delta && (s = fetch_jt(h->d_delta, delta, size_t(tot) * M)) != BVP_OK) return s;
    return BVP_OK;
}

void bvp_destroy(bvp_handle* h) {
    if (!h) return;
    DevBuf* devs[] = {&h->d_mesh, &h->d_h, &h->d_y, &h->d_ybak, &h->d_ybase, &h->d_K, &h->d_KI, &h->d_F,
                      &h->d_err, &h->d_inc, &h->d_iold, &h->d_Sb, &h->d_Rb, &h->d_rec, &h->d_tj, &h->d_hj,
                      &h->d_delta, &h->d_yj, &h->d_Fj, &h->d_scr, &h->d_iscr, &h->d_st, &h->d_order, &h->d_cap,
                      &h->d_node_off, &h->d_counter, &h->d_params, &h->d_params_j, &h->d_n_init,
                      &h->d_tspans, &h->d_y0, &h->d_y0_off, &h->d_out_off, &h->d_out_mesh,
                      &h->d_out_y, &h->d_out_K, &h->d_out_KI, &h->d_norm, &h->d_feat, &h->d_grid,
                      // the larger-state path's per-instance arrays
                      &h->d_bcres, &h->d_G, &h->d_lnorm, &h->d_lsq, &h->d_ldnorm, &h->d_lbad,
                      &h->d_active, &h->d_N, &h->d_newN,
                      // work-order tables and the error controllers' arrays
                      &h->d_inst_cost, &h->d_cost_tab, &h->d_gerr, &h->d_K_hi, &h->d_pause, &h->d_fx};
    for (DevBuf* b : devs)
        if (b->p) cudaFree(b->p);
    HostBuf* hosts[] = {&h->h_in, &h->h_st, &h->h_off, &h->h_mesh, &h->h_y, &h->h_K, &h->h_KI, &h->h_pause};
    for (HostBuf* b : hosts)
        if (b->p) cudaFreeHost(b->p);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->ev_in) cudaEventDestroy(h->ev_in);
    if (h->ev_side) cudaEventDestroy(h->ev_side);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->lib) cudaLibraryUnload(h->lib);
    if (h->lib_hi) cudaLibraryUnload(h->lib_hi);
    if (h->lib_blk) cudaLibraryUnload(h->lib_blk);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

}  // extern "C"
