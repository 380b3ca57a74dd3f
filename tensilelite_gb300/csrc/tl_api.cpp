// tl_api.cpp -- the C ABI (include/tensilelite.h) over the CUDA runtime.
//
// Host-side counterpart of TensileLite's L2/L3 harness: problem validation and solution choice
// (GemmMfmaSolver / GemmMfmaAsmSolution::generateKernel, src/gemmMfma.cpp:20-185), legality
// (checkKernelParameters, src/gemmMfmaKernelWriter.h:321-405), launch (StreamHip::Launch,
// ff_gpu_src/ff_hip_runtime.cpp:278-320) and the runtime's buffer calls (inc/ff_gpu.h:240-333).
// Unlike the reference, nothing here exits the process, launches are asynchronous on the caller's
// stream, and the runtime is a per-device handle rather than a global singleton.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "tl_internal.h"

struct tl_handle {
    int device = 0;
    int sm_count = 0;
    int cc_major = 0, cc_minor = 0;
    size_t smem_optin = 0;
    char name[256] = {0};
    int* d_err = nullptr;          // device error word
    double* d_norms = nullptr;     // error-norm scratch (3 doubles)
    float* d_amax = nullptr;       // fp8 amax scratch
    void* ws = nullptr;            // workspace: split-k partials, bf16x3 operands
    size_t ws_bytes = 0;
    int* counters = nullptr;       // split-k arrival counters (self-resetting)
    size_t counters_len = 0;
    int64_t launches = 0;
    uint64_t timeout_ns = 4000000000ull;
    unsigned long long* trace = nullptr;   // device timeline buffer (tl_set_trace), or null
    int64_t trace_bytes = 0;
    std::map<std::string, tl_gemm_solution> tuned;
    std::mutex mu;
    // Once a stream capture has recorded this handle's workspace address, a grown workspace retires
    // the old buffer here (freed by tl_destroy) instead of freeing it under a live graph.
    bool captured = false;
    std::vector<void*> retired;
    // Per-launch kernel timing: an event pair around each GEMM kernel launch, read back lazily.
    bool timing = false;
    std::vector<cudaEvent_t> tev;  // 2 * kTimingPairs events, start/stop interleaved
    size_t tev_used = 0;           // events recorded since the last fold
    double timing_ms = 0.0;
    int64_t timing_count = 0;
    // A planning handle (tl_init_host): a described device, no CUDA context use and no device
    // memory; only the planning calls accept it.
    bool host_only = false;
    int host_clusters4 = 0;        // clusters of 4 CTAs the described device runs at once (0: sm_count / 4)
};

struct tl_grouped_plan {
    tl_handle* h = nullptr;
    tl::TcGroupEntry* d_entries = nullptr;
    int4* d_units = nullptr;       // per work unit {problem, tile row, tile column, k-blocks}
    tl::TcGroupLaunch launch{};
    tl_gemm_solution sol{};
    double flops = 0.0;
};

struct tl_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct tl_timer {
    cudaEvent_t start = nullptr, stop = nullptr;
};

namespace tl {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

tl_status fail(tl_status st, const std::string& msg)
{
    g_last_error = msg;
    return st;
}

tl_status cuda_fail(cudaError_t e, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    g_last_error = m;
    return TL_ERR_CUDA;
}

namespace {

cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

bool is_split(int kernel) { return kernel == TL_KERNEL_BF16X3 || kernel == TL_KERNEL_BF16X6; }
int split_pieces(int kernel) { return kernel == TL_KERNEL_BF16X6 ? 3 : (kernel == TL_KERNEL_BF16X3 ? 2 : 1); }

std::string dims_str(const tl_gemm_problem& p)
{
    char buf[200];
    snprintf(buf, sizeof(buf), "m=%lld n=%lld k=%lld batch=%lld", (long long)p.m, (long long)p.n, (long long)p.k,
             (long long)p.batch);
    return buf;
}

// Basic validation shared by every path (sizes, leading dimensions, dtypes).
tl_status validate(const tl_gemm_problem* p)
{
    if (!p) return fail(TL_ERR_INVALID_ARG, "problem is NULL");
    if (p->m < 0 || p->n < 0 || p->k < 0 || p->batch < 1)
        return fail(TL_ERR_INVALID_ARG, "negative size or batch < 1: " + dims_str(*p));
    if (p->m > 0x7fffffffLL || p->n > 0x7fffffffLL || p->k > 0x7fffffffLL || p->batch > 65535)
        return fail(TL_ERR_UNSUPPORTED, "size beyond 2^31-1 (or batch > 65535): " + dims_str(*p));
    if (dtype_bytes(p->dtype_a) == 0 || dtype_bytes(p->dtype_d) == 0)
        return fail(TL_ERR_INVALID_ARG, "unknown dtype");
    if (p->dtype_a != p->dtype_b) return fail(TL_ERR_UNSUPPORTED, "dtype_a != dtype_b");
    if (p->dtype_c != p->dtype_d) return fail(TL_ERR_UNSUPPORTED, "dtype_c != dtype_d");
    if (p->dtype_d == TL_DTYPE_FP8_E4M3) {
        // E4M3 outputs come out of the tensor-core epilogue, with no C operand
        if (p->beta != 0.0f) return fail(TL_ERR_UNSUPPORTED, "an fp8 output takes beta == 0 (no fp8 C operand)");
        if (p->kernel == TL_KERNEL_SIMT) return fail(TL_ERR_UNSUPPORTED, "the CUDA-core kernel writes no fp8 output");
    }
    if (p->dtype_a == TL_DTYPE_FP32 && p->dtype_d != TL_DTYPE_FP32)
        return fail(TL_ERR_UNSUPPORTED, "fp32 inputs need an fp32 output");
    if ((p->trans_a != TL_OP_N && p->trans_a != TL_OP_T) || (p->trans_b != TL_OP_N && p->trans_b != TL_OP_T))
        return fail(TL_ERR_INVALID_ARG, "trans flags must be TL_OP_N or TL_OP_T");
    const int64_t a_rows = p->trans_a ? p->k : p->m;   // stored rows (leading dimension extent)
    const int64_t b_rows = p->trans_b ? p->n : p->k;
    if (p->lda < std::max<int64_t>(1, a_rows)) return fail(TL_ERR_INVALID_ARG, "lda smaller than op(A) storage rows");
    if (p->ldb < std::max<int64_t>(1, b_rows)) return fail(TL_ERR_INVALID_ARG, "ldb smaller than op(B) storage rows");
    if (p->ldd < std::max<int64_t>(1, p->m)) return fail(TL_ERR_INVALID_ARG, "ldd < m");
    if (p->beta != 0.0f && p->ldc < std::max<int64_t>(1, p->m)) return fail(TL_ERR_INVALID_ARG, "ldc < m");
    if (p->kernel < TL_KERNEL_AUTO || p->kernel > TL_KERNEL_BF16X6) return fail(TL_ERR_INVALID_ARG, "bad kernel id");
    if ((p->kernel == TL_KERNEL_BF16X3 || p->kernel == TL_KERNEL_BF16X6) && p->dtype_a != TL_DTYPE_FP32)
        return fail(TL_ERR_UNSUPPORTED, "bf16x3/bf16x6 need fp32 inputs");
    if (p->kernel == TL_KERNEL_TCGEN05 && p->dtype_a == TL_DTYPE_FP32)
        return fail(TL_ERR_UNSUPPORTED, "the tcgen05 kernel takes fp16/bf16/fp8 inputs (use BF16X3 for fp32)");
    if (p->out_rounding != TL_ROUND_RNE && p->out_rounding != TL_ROUND_TRUNCATE)
        return fail(TL_ERR_INVALID_ARG, "bad out_rounding");
    return TL_SUCCESS;
}

float scale_of(float s) { return s == 0.0f ? 1.0f : s; }

int tc_in_dtype(const tl_gemm_problem& p) { return p.dtype_a == TL_DTYPE_FP32 ? TL_DTYPE_BF16 : p.dtype_a; }

int row_elems(int in_dtype) { return kTcRowBytes / dtype_bytes(in_dtype); }

// Can TMA describe the operands as given?  (strides multiples of 16 bytes, 16-byte aligned bases)
bool tma_ok(const tl_gemm_problem& p, const void* A, const void* B, std::string* why)
{
    const int es = dtype_bytes(p.dtype_a);
    auto bad = [&](const char* w) { if (why) *why = w; return false; };
    if (is_split(p.kernel)) return true;   // operands are re-laid into the workspace
    if (!aligned16(A) || !aligned16(B)) return bad("A/B not 16-byte aligned");
    if ((p.lda * es) % 16 || (p.ldb * es) % 16) return bad("lda/ldb not a multiple of 16 bytes");
    if (p.batch > 1 && (((p.stride_a * es) % 16) || ((p.stride_b * es) % 16)))
        return bad("batch strides of A/B not multiples of 16 bytes");
    return true;
}

int resolve_kernel(const tl_gemm_problem& p)
{
    if (p.kernel != TL_KERNEL_AUTO) return p.kernel;
    return p.dtype_a == TL_DTYPE_FP32 ? TL_KERNEL_SIMT : TL_KERNEL_TCGEN05;
}

// Two CTA pairs per cluster sharing the m-side operand (macro_tile1 512) as a heuristic/tuner choice:
// on unless TL_CLUSTER4=0 in the environment (explicit solutions can always ask for it).
bool cluster4_enabled()
{
    static const bool on = [] {
        const char* e = getenv("TL_CLUSTER4");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Grouped plans order their problems by decreasing k unless TL_GROUP_ORDER=0 in the environment.
bool group_order_by_k()
{
    static const bool on = [] {
        const char* e = getenv("TL_GROUP_ORDER");
        return !(e && e[0] == '0');
    }();
    return on;
}

int max_stages(int bm_cta, size_t smem_optin)
{
    int s = kTcMaxStages;
    while (s > 2 && tc_smem_bytes(bm_cta, s) > smem_optin) --s;
    return s;
}

void simt_solution(tl_gemm_solution* s)
{
    memset(s, 0, sizeof(*s));
    s->kernel = TL_KERNEL_SIMT;
    s->macro_tile0 = 128;
    s->macro_tile1 = 128;
    s->depth_u = 8;
    s->stages = 2;
    s->wave_tile0 = 8;
    s->wave_tile1 = 8;
    s->split_k = 1;
}

bool m_mn_major(const tl_gemm_problem& p) { return p.trans_a == TL_OP_N; }   // A[m + k*lda]
bool n_mn_major(const tl_gemm_problem& p) { return p.trans_b == TL_OP_T; }   // B[n + k*ldb]

// NN problems on the tensor cores run as their transposed product D^T = B^T A^T (a TT problem:
// m and n, A and B exchanged) whose output the epilogue stores transposed, i.e. straight into the
// caller's column-major D.  An MN-major operand on the MMA's N side (the problem's m side: A of an
// NN problem) costs ~9 % at 4096^3 (NN and NT 1557 TFLOP/s against TN and TT 1700); on the M side
// it costs nothing, and the exchange puts it there.  Only for one GEMM (batch 1, the measured
// case), with beta == 0, k >= 2048 and without explicit split-k: the transposed epilogue reads C and finishes split tiles element by element
// across a warp, which measured slower than the exchange gains, and with short k its epilogue
// weighs more (4096 x 4096 x 1024: 31.4 against 30.5 us).  Not with a fused epilogue (its bias and amax
// follow the problem's m) nor fp8 (no MN-major fp8 operands).  TL_NN_TRANSPOSE=0 turns it off.
bool nn_view_enabled()
{
    static const bool on = [] {
        const char* e = getenv("TL_NN_TRANSPOSE");
        return !(e && e[0] == '0');
    }();
    return on;
}
bool tc_nn_view(const tl_gemm_problem& p, int kernel)
{
    return nn_view_enabled() && kernel == TL_KERNEL_TCGEN05 && p.trans_a == TL_OP_N && p.trans_b == TL_OP_N &&
           p.beta == 0.0f && p.k >= 2048 && p.batch == 1 && (p.dtype_a == TL_DTYPE_FP16 || p.dtype_a == TL_DTYPE_BF16) &&
           p.dtype_d != TL_DTYPE_FP8_E4M3;
}
// The kernel's view of an NN problem: C, D, their leading dimensions and strides stay the caller's.
tl_gemm_problem nn_view(const tl_gemm_problem& p)
{
    tl_gemm_problem q = p;
    q.m = p.n;
    q.n = p.m;
    q.trans_a = TL_OP_T;
    q.trans_b = TL_OP_T;
    q.lda = p.ldb;
    q.ldb = p.lda;
    q.stride_a = p.stride_b;
    q.stride_b = p.stride_a;
    return q;
}
void tc_heuristic(const tl_handle* h, const tl_gemm_problem& p, int kernel, tl_gemm_solution* s);
// A view's solution without explicit split-k keeps the view.
bool view_solution_ok(const tl_gemm_solution& s) { return s.split_k <= 1; }
// The heuristic for a problem that may run as its view: the view's pick when it needs no split-k,
// else the caller's problem's pick (*view reports which).
void tc_heuristic_viewed(const tl_handle* h, const tl_gemm_problem& p, int kernel, bool allow, tl_gemm_solution* s,
                         bool* view)
{
    *view = false;
    if (allow && tc_nn_view(p, kernel)) {
        tc_heuristic(h, nn_view(p), kernel, s);
        if (view_solution_ok(*s)) {
            *view = true;
            return;
        }
    }
    tc_heuristic(h, p, kernel, s);
}

// Two CTA pairs per cluster (macro_tile1 512) load the shared m-side operand with a TMA multicast
// copy.  That copy is kept to memory of the GPU running the kernel: an operand must be device (or
// managed) memory of `device`, as cudaPointerGetAttributes reports it -- not host memory, another
// GPU's memory or an unregistered pointer.
bool on_device(const void* ptr, int device)
{
    if (!ptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == device;
}

bool multicast_ok(const void* A, const void* B, int device) { return on_device(A, device) && on_device(B, device); }

tl_status multicast_refused()
{
    return fail(TL_ERR_UNSUPPORTED,
                "macro_tile1 512 (two CTA pairs sharing the m-side operand) uses a TMA multicast load, which this "
                "library runs only on device memory of the current GPU; A or B is host memory, another device's "
                "memory or not a CUDA allocation (use macro_tile1 256)");
}

// The heuristic's tile without the multicast variant: the same tile on a CTA pair.
void drop_cluster4(const tl_handle* h, tl_gemm_solution* s);

tl_status check_tc_solution(const tl_handle* h, const tl_gemm_problem& p, const tl_gemm_solution& s);

// Modelled duration of one tensor-core launch, in SM clocks.  Per 128-byte k-block a CTA needs its
// MMA issue time plus a cost per operand byte it stages (below) -- so a CTA pair or two pairs
// sharing the m-side operand (fewer bytes per SM) win even on a partial wave.
// Tiles run in persistent waves; a last wave that would leave half the workers idle is split along
// k as the launch does; a tile's epilogue overlaps the next tile's main loop unless it is longer.
double tc_cost(const tl_handle* h, const tl_gemm_problem& p, const tl_gemm_solution& s, int in_dtype)
{
    const int W = row_elems(in_dtype);
    const int cg = s.macro_tile1 / kTcTileN;
    const int bm = s.macro_tile0;
    const int64_t num_kb = std::max<int64_t>(1, (p.k + W - 1) / W);
    const int64_t tiles = ((p.n + kTcTileN * cg - 1) / (kTcTileN * cg)) * ((p.m + bm - 1) / bm) * p.batch;
    // real devices: the co-resident cluster count (clusters of 4 leave some SMs idle)
    const int64_t workers = std::max<int64_t>(
        1, h->d_err ? tc_workers(in_dtype, p.dtype_d, cg, bm, s.stages, h->sm_count)
                    : (cg == 4 && h->host_clusters4 > 0 ? h->host_clusters4 : h->sm_count / cg));
    const int64_t split = std::max<int64_t>(1, s.split_k);
    const int64_t units = tiles * split;
    // per k-block and CTA: the MMA issue time (4 MMAs; about 500 clocks for any width up to 128
    // columns, 716 for 256) plus a cost per staged operand byte that grows with the number of SMs
    // loading at once -- fitted to the per-k-block times measured on GB300 for one SM / a pair,
    // 128 / 256 columns (690-1000 clocks with every SM busy)
    const double mma_kb = std::max(716.0 * bm / 256.0, 500.0);
    const double bytes_kb = static_cast<double>(kTcTileN) * kTcRowBytes + static_cast<double>(bm) / cg * kTcRowBytes;
    auto per_kb = [&](double active_ctas) {
        const double load = std::max(0.5, std::min(1.0, active_ctas / h->sm_count));
        return mma_kb + bytes_kb * 0.0068 * load;
    };
    const int out_b = dtype_bytes(p.dtype_d);
    // each CTA drains a 128 x bm accumulator (a pair's MMA is 256 x bm)
    const double epi = static_cast<double>(kTcTileN) * bm * (out_b + (p.beta != 0.0f ? out_b : 0)) / 27.0;
    auto unit_time = [&](double kb, double active_ctas) { return std::max(kb * per_kb(active_ctas), epi) + 1500.0; };
    const double kb_unit = static_cast<double>(num_kb) / split;
    const int64_t full = units / workers, rem = units % workers;
    double cost = 6000.0 + epi;      // launch, prologue, the last tile's epilogue
    cost += static_cast<double>(full) * unit_time(kb_unit, static_cast<double>(std::min(units, workers)) * cg);
    if (rem > 0) {
        const int64_t R = rem * num_kb;
        const int64_t Wb = std::min<int64_t>(std::min<int64_t>(workers, 8 * rem), R / 2);
        int64_t S = std::min<int64_t>(std::min<int64_t>(workers / rem, num_kb / 16), 8);
        if (s.tail_split > 1) S = std::min<int64_t>(s.tail_split, num_kb);
        if (split == 1 && Wb > 1 && Wb >= rem && s.promote_k == 0 &&
            (s.tail_split == -1 || (s.tail_split == 0 && R / Wb >= 48))) {
            // balanced split of the last partial wave (reduction exposed without a whole wave after)
            cost += unit_time(std::ceil(static_cast<double>(R) / Wb), static_cast<double>(workers * cg)) +
                    (full >= 1 ? 1000.0 : 3000.0 + epi);
        } else if (split == 1 && s.tail_split != 1 && s.tail_split != -1 && tiles > workers && 2 * rem <= workers &&
                   S >= 2) {
            cost += unit_time(static_cast<double>(num_kb) / S, static_cast<double>(rem * S * cg)) + 2000.0 + epi;
        } else {
            cost += unit_time(kb_unit, static_cast<double>(rem * cg));
        }
    }
    if (split > 1) {
        // every split parks a fp32 partial; with all split units resident the splits reduce a share
        // each (parallel), else the last to arrive reads all of them
        const double part = static_cast<double>(kTcTileN) * bm * 4.0 / 27.0;
        if (units <= workers) cost += 1500.0 + part + (part * split + epi) / split;
        else cost += 3000.0 + part + part * split + epi;
        // a CTA pair's split epilogue (remote TMEM hand-backs, both CTAs parking) measured ~0.7 us
        // longer than one CTA's on bf16 480 x 1024 x 4096 at split-k 4
        if (cg >= 2) cost += 1400.0;
    }
    return cost;
}

void tc_heuristic(const tl_handle* h, const tl_gemm_problem& p, int kernel, tl_gemm_solution* s)
{
    memset(s, 0, sizeof(*s));
    s->kernel = kernel;
    const int in = is_split(kernel) ? TL_DTYPE_BF16 : p.dtype_a;
    const int W = row_elems(in);
    const int64_t tiles_n = (p.n + kTcTileN - 1) / kTcTileN;
    const int64_t num_kb = (p.k + W - 1) / W;
    s->depth_u = W;
    // operands of up to ~64 MB stay L2-resident, where linear tile order measured best
    const int64_t op_bytes = (p.m * p.k + p.n * p.k) * dtype_bytes(in);
    s->raster = (tiles_n > 8 && op_bytes > (int64_t(96) << 20)) ? 8 : 0;
    if (is_split(kernel)) {
        // FP32-accurate paths: 128-wide tiles so the dominant product can be promoted out of TMEM
        // every 256 k (the chain length sets the tensor-core accumulation error)
        s->macro_tile0 = 128;
        s->promote_k = 256;
        const int64_t t128 = tiles_n * ((p.m + 127) / 128) * p.batch;
        int split = 1;
        if (t128 < h->sm_count / 2 && num_kb >= 8)
            split = std::max(1, static_cast<int>(std::min<int64_t>(std::min<int64_t>(h->sm_count / std::max<int64_t>(1, t128),
                                                                                     num_kb / 4), 16)));
        s->split_k = split;
        // a CTA pair per 256 x 128 tile (half the m-side operand per SM): measured 6 % faster at 8192^3
        s->macro_tile1 = 2 * kTcTileN;
        s->stages = std::min(6, max_stages(64, h->smem_optin));
        if (check_tc_solution(h, p, *s) != TL_SUCCESS) {
            s->macro_tile1 = kTcTileN;
            s->stages = std::min(6, max_stages(128, h->smem_optin));
        }
        return;
    }
    // the legal tile with the least modelled time
    double best = 0.0;
    bool have = false;
    tl_gemm_solution c = *s;
    for (int cg : {4, 2, 1})
        for (int bm : {256, 128, 192, 64})
            for (int split : {1, 2, 3, 4, 6, 8, 12, 16}) {
                if (cg == 4 && !cluster4_enabled()) continue;
                if (split > 1 && (split > num_kb / 2 || split > 16)) continue;
                c.macro_tile0 = bm;
                c.macro_tile1 = kTcTileN * cg;
                // measured on GB300: beyond ~6 stages (about 190 KB in flight) a deeper ring gains nothing
                c.stages = std::min(6, max_stages(bm / (cg >= 2 ? 2 : 1), h->smem_optin));
                c.split_k = split;
                c.tail_split = 0;
                if (check_tc_solution(h, p, c) != TL_SUCCESS) continue;
                const double cost = tc_cost(h, p, c, in) * (split > 1 ? 1.0 + 0.02 * split : 1.0);
                if (!have || cost < best * 0.995) {
                    best = cost;
                    *s = c;
                    have = true;
                }
            }
    if (!have) {
        // nothing legal (the caller's check reports why): a plain one-SM tile
        s->macro_tile0 = 128;
        s->macro_tile1 = kTcTileN;
        s->stages = std::min(6, max_stages(128, h->smem_optin));
        s->split_k = 1;
    }
    s->wave_tile0 = 0;
    s->wave_tile1 = 0;
    s->ctas = 0;
}

tl_status check_tc_solution(const tl_handle* h, const tl_gemm_problem& p, const tl_gemm_solution& s)
{
    const int in = is_split(s.kernel) ? TL_DTYPE_BF16 : p.dtype_a;
    if (in != TL_DTYPE_FP16 && in != TL_DTYPE_BF16 && in != TL_DTYPE_FP8_E4M3)
        return fail(TL_ERR_UNSUPPORTED, "tcgen05 kernel needs fp16, bf16 or fp8 operands");
    const int W = row_elems(in);
    if (s.macro_tile1 != kTcTileN && s.macro_tile1 != 2 * kTcTileN && s.macro_tile1 != 4 * kTcTileN)
        return fail(TL_ERR_UNSUPPORTED, "macro_tile1 (n) must be 128 (one SM), 256 (a CTA pair) or 512 (two pairs "
                                        "sharing the m-side operand) for tcgen05");
    const int cg = s.macro_tile1 / kTcTileN;
    const int cta_group = cg >= 2 ? 2 : 1;
    const int bm = s.macro_tile0;
    if (bm != 64 && bm != 128 && bm != 192 && bm != 256)
        return fail(TL_ERR_UNSUPPORTED, "macro_tile0 (m) must be 64, 128, 192 or 256");
    if (cg == 2 && bm != 128 && bm != 256)
        return fail(TL_ERR_UNSUPPORTED, "a CTA pair (macro_tile1 256) needs macro_tile0 128 or 256");
    if (cg == 4 && (bm != 256 || s.promote_k > 0 || is_split(s.kernel)))
        return fail(TL_ERR_UNSUPPORTED, "two CTA pairs (macro_tile1 512) need macro_tile0 256 and no promotion");
    if (cg == 4 && m_mn_major(p) && bm / 2 != 2 * W)
        return fail(TL_ERR_UNSUPPORTED, "two CTA pairs with MN-major A need two 128-byte chunks of m per CTA");
    const bool mmn = m_mn_major(p);
    if (mmn && (bm / cta_group) % W)
        return fail(TL_ERR_UNSUPPORTED, "m rows per CTA must be a multiple of the 128-byte row for MN-major A");
    if (s.depth_u != 0 && s.depth_u != W) return fail(TL_ERR_UNSUPPORTED, "depth_u is fixed to one 128-byte row");
    if (s.stages < 2 || s.stages > kTcMaxStages) return fail(TL_ERR_UNSUPPORTED, "stages must be in [2, 8]");
    if (tc_smem_bytes(bm / cta_group, s.stages) > h->smem_optin)
        return fail(TL_ERR_UNSUPPORTED, "shared memory budget exceeded");
    const int64_t num_kb = (p.k + W - 1) / W;
    if (s.split_k < 1 || (num_kb > 0 && s.split_k > num_kb) || s.split_k > 64)
        return fail(TL_ERR_UNSUPPORTED, "split_k must be in [1, min(64, k blocks)]");
    if (s.raster < 0 || s.ctas < 0) return fail(TL_ERR_INVALID_ARG, "raster and ctas must be >= 0");
    if (s.promote_k < 0) return fail(TL_ERR_INVALID_ARG, "promote_k must be >= 0");
    if (s.tail_split < -1 || s.tail_split > 8) return fail(TL_ERR_INVALID_ARG, "tail_split must be in [-1, 8]");
    if (s.promote_k > 0 && bm != 128)
        return fail(TL_ERR_UNSUPPORTED, "promote_k needs macro_tile0 == 128 (fp32 running sums, TMEM budget)");
    if (s.debug_flags & ~TL_DEBUG_SKIP_LOADS) return fail(TL_ERR_INVALID_ARG, "unknown debug_flags bit");
    return TL_SUCCESS;
}

void drop_cluster4(const tl_handle* h, tl_gemm_solution* s)
{
    if (s->macro_tile1 != 4 * kTcTileN) return;
    s->macro_tile1 = 2 * kTcTileN;
    s->stages = std::min(6, max_stages(s->macro_tile0 / 2, h->smem_optin));
}

std::string problem_key(const tl_handle* h, const tl_gemm_problem& p)
{
    char buf[400];
    snprintf(buf, sizeof(buf), "%s|sm%d%d|a%d|d%d|k%d|%c%c|%lld|%lld|%lld|%lld|%lld|%lld", h->name, h->cc_major,
             h->cc_minor, p.dtype_a, p.dtype_d, p.kernel, p.trans_a ? 'T' : 'N', p.trans_b ? 'T' : 'N', (long long)p.m,
             (long long)p.n, (long long)p.k, (long long)p.batch, (long long)p.lda, (long long)p.ldb);
    for (char* c = buf; *c; ++c)
        if (*c == '"' || *c == '\\') *c = '_';
    return buf;
}

// Set for the calling thread while tl_gemm runs on a stream that is being captured: buffers may not
// grow then (an allocation is not capturable, and the graph would keep the old address).
static thread_local bool t_capturing = false;

tl_status grow_refused_in_capture(const char* what)
{
    return fail(TL_ERR_UNSUPPORTED, std::string(what) + " would have to grow during stream capture: run the same "
                                    "problem once on this handle outside the capture first");
}

void retire_or_free(tl_handle* h, void* ptr)
{
    cudaDeviceSynchronize();
    if (h->captured) h->retired.push_back(ptr);
    else cudaFree(ptr);
}

tl_status ensure_ws(tl_handle* h, size_t bytes)
{
    if (bytes <= h->ws_bytes) return TL_SUCCESS;
    if (t_capturing) return grow_refused_in_capture("the workspace");
    if (h->ws) {
        retire_or_free(h, h->ws);
        h->ws = nullptr;
        h->ws_bytes = 0;
    }
    size_t want = std::max<size_t>(bytes, 1 << 20);
    cudaError_t e = cudaMalloc(&h->ws, want);
    if (e != cudaSuccess) return fail(TL_ERR_ALLOC, "workspace allocation failed");
    h->ws_bytes = want;
    return TL_SUCCESS;
}

tl_status ensure_counters(tl_handle* h, size_t n)
{
    if (n <= h->counters_len) return TL_SUCCESS;
    if (t_capturing) return grow_refused_in_capture("the split-k counter array");
    if (h->counters) {
        retire_or_free(h, h->counters);
        h->counters = nullptr;
        h->counters_len = 0;
    }
    size_t want = std::max<size_t>(n, 4096);
    if (cudaMalloc(&h->counters, want * sizeof(int)) != cudaSuccess) return fail(TL_ERR_ALLOC, "counter allocation failed");
    if (cudaMemset(h->counters, 0, want * sizeof(int)) != cudaSuccess) return fail(TL_ERR_CUDA, "counter memset failed");
    h->counters_len = want;
    return TL_SUCCESS;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// The driver-API calls (tensor-map encoding) need the device's primary context current on the calling
// thread; a thread that has only made runtime calls so far (e.g. an autograd worker) may not have it.
// cudaSetDevice on the already-current device binds it.  Once per thread and device.
tl_status bind_thread(const tl_handle* h)
{
    static thread_local int bound = -1;
    if (bound == h->device) return TL_SUCCESS;
    int cur = -1;
    TL_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != h->device)
        return fail(TL_ERR_INVALID_ARG, "handle belongs to device " + std::to_string(h->device) +
                                            " but the current device is " + std::to_string(cur));
    TL_CUDA_TRY(cudaSetDevice(cur));
    bound = cur;
    return TL_SUCCESS;
}

// Everything a GEMM launch needs once the solution is fixed; preparing allocates, enqueueing
// only launches (so enqueue can be captured in a CUDA graph).
struct Prepared {
    tl_gemm_problem p;
    tl_gemm_solution s;
    int kernel;
    void* D;
    const void* C;
    const void* A;
    const void* B;
    // split-precision operand pieces in the workspace (bf16x3: 2 per operand, bf16x6: 3)
    uint16_t* a_pc[3] = {nullptr, nullptr, nullptr};
    uint16_t* b_pc[3] = {nullptr, nullptr, nullptr};
    int64_t a_span = 0, b_span = 0;
    float* ws_partials = nullptr;
    size_t part_bytes = 0;
    tl_epilogue epi{};
    bool epi_on = false;
    bool tview = false;      // p is the transposed view of the caller's NN problem (tc_nn_view)
};

int64_t operand_span(int64_t ld, int64_t cols, int64_t batch, int64_t bstride, int64_t rows)
{
    if (rows == 0 || cols == 0) return 0;
    return (batch - 1) * bstride + (cols - 1) * ld + rows;
}

tl_status prepare(tl_handle* h, const tl_gemm_problem* prob, const tl_gemm_solution* sol, void* D, const void* C,
                  const void* A, const void* B, Prepared* out, bool epilogue = false)
{
    tl_status st = bind_thread(h);
    if (st != TL_SUCCESS) return st;
    st = validate(prob);
    if (st != TL_SUCCESS) return st;
    Prepared& P = *out;
    P.p = *prob;
    P.D = D; P.C = C; P.A = A; P.B = B;
    const tl_gemm_problem& p = P.p;
    if ((p.m && p.n) && !D) return fail(TL_ERR_INVALID_ARG, "D is NULL");
    if (p.beta != 0.0f && !C && p.m && p.n) return fail(TL_ERR_INVALID_ARG, "C is NULL with beta != 0");
    if (p.k > 0 && p.m > 0 && p.n > 0 && (!A || !B)) return fail(TL_ERR_INVALID_ARG, "A or B is NULL");

    int kernel = resolve_kernel(p);
    bool view = false;
    if (sol) {
        P.s = *sol;
        if (P.s.kernel == TL_KERNEL_AUTO) P.s.kernel = kernel;
        kernel = P.s.kernel;
        if (p.kernel != TL_KERNEL_AUTO && kernel != p.kernel)
            return fail(TL_ERR_INVALID_ARG, "solution kernel differs from the problem's kernel request");
        view = !epilogue && tc_nn_view(p, kernel) && view_solution_ok(P.s);
    } else {
        std::lock_guard<std::mutex> g(h->mu);
        auto it = h->tuned.find(problem_key(h, p));
        if (it != h->tuned.end()) {
            P.s = it->second;
            kernel = P.s.kernel;
            view = !epilogue && tc_nn_view(p, kernel) && view_solution_ok(P.s);
        } else if (kernel == TL_KERNEL_SIMT) {
            simt_solution(&P.s);
        } else {
            tc_heuristic_viewed(h, p, kernel, !epilogue, &P.s, &view);
        }
    }
    // an NN problem runs as its transposed view from here on (solutions are for the view)
    if (view) {
        P.p = nn_view(*prob);
        P.A = B;
        P.B = A;
        A = P.A;
        B = P.B;
        P.tview = true;
    }
    // operands the TMA cannot describe fall back to the SIMT kernel when the caller left it to us
    std::string why;
    const bool has_work = p.m > 0 && p.n > 0 && p.k > 0;
    if (kernel == TL_KERNEL_TCGEN05 && has_work && !tma_ok(p, A, B, &why)) {
        if (p.kernel == TL_KERNEL_AUTO && !sol && p.dtype_d != TL_DTYPE_FP8_E4M3) {
            kernel = TL_KERNEL_SIMT;
            simt_solution(&P.s);
            if (P.tview) {            // the CUDA-core kernel takes the caller's problem as it is
                P.p = *prob;
                P.A = B;
                P.B = A;
                P.tview = false;
            }
        } else {
            return fail(TL_ERR_UNSUPPORTED, "tcgen05 kernel: " + why);
        }
    }
    // the multicast variant reads A and B only where they are this GPU's own memory: an explicit
    // request is refused otherwise, a heuristic or tuned choice drops to the CTA pair
    if (kernel == TL_KERNEL_TCGEN05 && has_work && P.s.macro_tile1 == 4 * kTcTileN && !multicast_ok(A, B, h->device)) {
        if (sol) return multicast_refused();
        drop_cluster4(h, &P.s);
    }
    P.kernel = kernel;
    if (kernel == TL_KERNEL_SIMT) {
        if (P.s.macro_tile0 != 128 || P.s.macro_tile1 != 128 || (P.s.depth_u && P.s.depth_u != 8) ||
            (P.s.split_k > 1))
            return fail(TL_ERR_UNSUPPORTED, "SIMT kernel supports macro tile 128x128, depth_u 8, split_k 1");
        return TL_SUCCESS;
    }
    if (kernel == TL_KERNEL_TCGEN05 && p.dtype_a == TL_DTYPE_FP32)
        return fail(TL_ERR_UNSUPPORTED, "tcgen05 kernel needs fp16/bf16/fp8 inputs");
    if (is_split(kernel) && p.dtype_a != TL_DTYPE_FP32)
        return fail(TL_ERR_UNSUPPORTED, "bf16x3/bf16x6 need fp32 inputs");
    if ((st = check_tc_solution(h, p, P.s)) != TL_SUCCESS) return st;
    if (p.m == 0 || p.n == 0 || p.k == 0) return TL_SUCCESS;

    // workspace: [split pieces of A][split pieces of B][split-k partials]
    size_t need = 0;
    size_t off_a[3] = {0, 0, 0}, off_b[3] = {0, 0, 0}, off_part = 0;
    const int npc = split_pieces(kernel);
    if (is_split(kernel)) {
        const int64_t a_rows = p.trans_a ? p.k : p.m, a_cols = p.trans_a ? p.m : p.k;
        const int64_t b_rows = p.trans_b ? p.n : p.k, b_cols = p.trans_b ? p.k : p.n;
        P.a_span = operand_span(p.lda, a_cols, p.batch, p.stride_a, a_rows);
        P.b_span = operand_span(p.ldb, b_cols, p.batch, p.stride_b, b_rows);
        for (int i = 0; i < npc; ++i) { off_a[i] = need; need = align_up(need + P.a_span * 2, 256); }
        for (int i = 0; i < npc; ++i) { off_b[i] = need; need = align_up(need + P.b_span * 2, 256); }
    }
    const int W = row_elems(tc_in_dtype(p));
    (void)W;
    const int cgp = P.s.macro_tile1 / kTcTileN;
    const int64_t tiles = ((p.n + kTcTileN * cgp - 1) / (kTcTileN * cgp)) * cgp *
                          ((p.m + P.s.macro_tile0 - 1) / P.s.macro_tile0) * p.batch;
    if (P.s.split_k > 1) {
        off_part = need;
        P.part_bytes = static_cast<size_t>(tiles) * P.s.split_k * kTcTileN * P.s.macro_tile0 * sizeof(float);
        need = off_part + P.part_bytes;
        if ((st = ensure_counters(h, static_cast<size_t>(tiles))) != TL_SUCCESS) return st;
    } else if (P.s.tail_split != 1) {
        // a split last wave: at most one tile per SM is split; an explicit tail split S keeps S
        // partial slabs per tile, the automatic balanced split up to three (fewer, longer pieces
        // are chosen at launch when a tile would need more)
        off_part = need;
        P.part_bytes = static_cast<size_t>(h->sm_count) * kTcTileN * P.s.macro_tile0 * sizeof(float) *
                       static_cast<size_t>(P.s.tail_split > 1 ? P.s.tail_split : (P.s.tail_split == -1 ? 9 : 3));
        need = off_part + P.part_bytes;
        if ((st = ensure_counters(h, static_cast<size_t>(h->sm_count))) != TL_SUCCESS) return st;
    }
    if (need) {
        if ((st = ensure_ws(h, need)) != TL_SUCCESS) return st;
        char* base = static_cast<char*>(h->ws);
        if (is_split(kernel)) {
            for (int i = 0; i < npc; ++i) {
                P.a_pc[i] = reinterpret_cast<uint16_t*>(base + off_a[i]);
                P.b_pc[i] = reinterpret_cast<uint16_t*>(base + off_b[i]);
            }
        }
        if (P.part_bytes) P.ws_partials = reinterpret_cast<float*>(base + off_part);
    }
    if (is_split(kernel)) {
        // the split copies keep the caller's leading dimensions; TMA needs them 16-byte aligned in bf16
        if ((p.lda * 2) % 16 || (p.ldb * 2) % 16 || (p.batch > 1 && ((p.stride_a * 2) % 16 || (p.stride_b * 2) % 16)))
            return fail(TL_ERR_UNSUPPORTED, "bf16x3/bf16x6: lda/ldb (and batch strides) must be multiples of 8 elements");
    }
    return TL_SUCCESS;
}

constexpr size_t kTimingPairs = 1024;

// Adds the elapsed times of every recorded start/stop pair to the running sum (waits for the last stop).
tl_status timing_fold(tl_handle* h)
{
    if (h->tev_used == 0) return TL_SUCCESS;
    TL_CUDA_TRY(cudaEventSynchronize(h->tev[h->tev_used - 1]));
    for (size_t i = 0; i + 1 < h->tev_used; i += 2) {
        float ms = 0.0f;
        TL_CUDA_TRY(cudaEventElapsedTime(&ms, h->tev[i], h->tev[i + 1]));
        h->timing_ms += ms;
        h->timing_count += 1;
    }
    h->tev_used = 0;
    return TL_SUCCESS;
}

bool stream_capturing(cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

// Records the start event of a timed launch; returns false when timing is off (or the stream is being
// captured, where an event record would become a graph node instead of a timestamp).
bool timing_begin(tl_handle* h, cudaStream_t s)
{
    if (!h->timing || h->tev.empty() || stream_capturing(s)) return false;
    if (h->tev_used + 2 > h->tev.size() && timing_fold(h) != TL_SUCCESS) return false;
    return cudaEventRecord(h->tev[h->tev_used], s) == cudaSuccess;
}

void timing_end(tl_handle* h, cudaStream_t s, bool started, tl_status launch_status)
{
    if (!started) return;
    if (launch_status == TL_SUCCESS && cudaEventRecord(h->tev[h->tev_used + 1], s) == cudaSuccess)
        h->tev_used += 2;
}

tl_status enqueue(tl_handle* h, const Prepared& P, cudaStream_t s)
{
    const tl_gemm_problem& p = P.p;
    if (p.m == 0 || p.n == 0) return TL_SUCCESS;
    const float alpha = p.alpha * scale_of(p.scale_a) * scale_of(p.scale_b);
    if (p.k == 0 || alpha == 0.0f) {
        return aux_scale_c(p.dtype_d, p.out_rounding, P.D, p.ldd, p.stride_d, P.C, p.ldc, p.stride_c, p.m, p.n,
                           p.batch, p.beta, s, &h->launches);
    }
    if (P.kernel == TL_KERNEL_SIMT) {
        SimtLaunch L;
        L.a_dtype = p.dtype_a; L.out_dtype = p.dtype_d; L.out_trunc = p.out_rounding;
        L.trans_a = p.trans_a; L.trans_b = p.trans_b;
        L.M = p.m; L.N = p.n; L.K = p.k; L.batch = p.batch;
        L.A = P.A; L.B = P.B; L.C = P.C; L.D = P.D;
        L.lda = p.lda; L.ldb = p.ldb; L.ldc = p.ldc; L.ldd = p.ldd;
        L.sa = p.stride_a; L.sb = p.stride_b; L.sc = p.stride_c; L.sd = p.stride_d;
        L.alpha = alpha; L.beta = p.beta;
        const bool timed = timing_begin(h, s);
        const tl_status st = simt_gemm_launch(L, s, &h->launches);
        timing_end(h, s, timed, st);
        return st;
    }
    TcLaunch L;
    memset(&L, 0, sizeof(L));
    L.in_dtype = tc_in_dtype(p);
    L.out_dtype = p.dtype_d;
    L.out_trunc = p.out_rounding;
    L.pieces = split_pieces(P.kernel);
    const void* Apc[3] = {P.A, nullptr, nullptr};
    const void* Bpc[3] = {P.B, nullptr, nullptr};
    if (L.pieces > 1) {
        const int64_t a_rows = p.trans_a ? p.k : p.m, a_cols = p.trans_a ? p.m : p.k;
        const int64_t b_rows = p.trans_b ? p.n : p.k, b_cols = p.trans_b ? p.k : p.n;
        tl_status st = aux_split_bf16(static_cast<const float*>(P.A), a_rows, a_cols, p.lda, p.batch, p.stride_a,
                                      P.a_pc[0], P.a_pc[1], P.a_pc[2], s, &h->launches);
        if (st != TL_SUCCESS) return st;
        st = aux_split_bf16(static_cast<const float*>(P.B), b_rows, b_cols, p.ldb, p.batch, p.stride_b, P.b_pc[0],
                            P.b_pc[1], P.b_pc[2], s, &h->launches);
        if (st != TL_SUCCESS) return st;
        for (int i = 0; i < L.pieces; ++i) {
            Apc[i] = P.a_pc[i];
            Bpc[i] = P.b_pc[i];
        }
    }
    for (int i = 0; i < L.pieces; ++i) {
        L.opM[i] = {Apc[i], p.m, p.lda, p.stride_a, m_mn_major(p) ? 1 : 0};
        L.opN[i] = {Bpc[i], p.n, p.ldb, p.stride_b, n_mn_major(p) ? 1 : 0};
    }
    L.M = p.m; L.N = p.n; L.K = p.k; L.batch = p.batch;
    L.D = P.D; L.C = (p.beta != 0.0f) ? P.C : nullptr;
    L.ldd = p.ldd; L.ldc = p.ldc; L.stride_d = p.stride_d; L.stride_c = p.stride_c;
    L.alpha = alpha; L.beta = p.beta;
    L.bm = P.s.macro_tile0;
    L.stages = P.s.stages;
    L.split_k = P.s.split_k;
    L.raster = P.s.raster;
    L.ctas = P.s.ctas;
    L.promote_k = P.s.promote_k;
    L.cg = P.s.macro_tile1 / kTcTileN;
    L.err = h->d_err;
    L.timeout_ns = h->timeout_ns;
    L.trace = h->trace;
    L.trace_bytes = h->trace_bytes;
    L.workspace = P.ws_partials;
    L.workspace_bytes = P.part_bytes;
    L.counters = h->counters;
    L.counters_len = h->counters_len;
    L.tail_split = P.s.tail_split;
    L.sm_count = h->sm_count;
    // fp8 outputs are written by the fused-epilogue kernels (no bias or activation unless asked for)
    L.epi_on = (P.epi_on || p.dtype_d == TL_DTYPE_FP8_E4M3) ? 1 : 0;
    L.epi_dscale = (P.epi_on && P.epi.d_scale != 0.0f) ? P.epi.d_scale : 1.0f;
    L.epi_bias = P.epi.bias;
    L.epi_amax = P.epi.amax;
    L.epi_bias_dtype = P.epi.bias_dtype;
    L.epi_act = P.epi.activation;
    L.debug_flags = P.s.debug_flags;
    L.out_t = P.tview ? 1 : 0;
    const bool timed = timing_begin(h, s);
    const tl_status st = tc_gemm_launch(L, s, &h->launches);
    timing_end(h, s, timed, st);
    return st;
}

// ---- tuner ------------------------------------------------------------------------------------------
std::vector<tl_gemm_solution> tc_candidates(const tl_handle* h, const tl_gemm_problem& p, int kernel)
{
    std::vector<std::pair<double, tl_gemm_solution>> ranked;
    const int in = is_split(kernel) ? TL_DTYPE_BF16 : p.dtype_a;
    const int W = row_elems(in);
    const int64_t num_kb = std::max<int64_t>(1, (p.k + W - 1) / W);
    const int64_t tiles_n = (p.n + kTcTileN - 1) / kTcTileN;
    for (int cg : {1, 2, 4})
    for (int bm : {64, 128, 192, 256}) {
        for (int split : {1, 2, 3, 4, 6, 8, 12, 16}) {
            if (cg == 4 && !cluster4_enabled()) continue;
            if (split > num_kb) continue;
            for (int raster : {0, 4, 8, 16}) {
                tl_gemm_solution s;
                memset(&s, 0, sizeof(s));
                s.kernel = kernel;
                s.macro_tile0 = bm;
                s.macro_tile1 = kTcTileN * cg;
                s.depth_u = W;
                s.stages = max_stages(bm / (cg >= 2 ? 2 : 1), h->smem_optin);
                s.split_k = split;
                s.raster = raster;
                if (is_split(kernel)) s.promote_k = 256;
                if (raster && raster >= tiles_n) continue;
                if (check_tc_solution(h, p, s) != TL_SUCCESS) continue;
                double cost = tc_cost(h, p, s, in) * (split > 1 ? 1.0 + 0.02 * split : 1.0);
                if (raster == 0 && tiles_n > 8) cost *= 1.02;
                ranked.push_back({cost, s});
            }
        }
    }
    std::stable_sort(ranked.begin(), ranked.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    std::vector<tl_gemm_solution> out;
    for (auto& r : ranked) out.push_back(r.second);
    return out;
}

tl_status save_cache(const char* path, const std::string& key, const tl_gemm_solution& s, float ms)
{
    // line-oriented JSON object:
    //   "key": [kernel, mt0, mt1, du, stages, wt0, wt1, split, raster, ctas, promote_k, tail_split, ms]
    std::map<std::string, std::string> lines;
    {
        std::ifstream in(path);
        std::string line;
        while (std::getline(in, line)) {
            size_t q0 = line.find('"');
            size_t q1 = line.find("\":", q0 + 1);
            if (q0 == std::string::npos || q1 == std::string::npos) continue;
            std::string k = line.substr(q0 + 1, q1 - q0 - 1);
            std::string v = line.substr(q1 + 2);
            while (!v.empty() && (v.back() == ',' || v.back() == ' ' || v.back() == '\r')) v.pop_back();
            lines[k] = v;
        }
    }
    char buf[256];
    snprintf(buf, sizeof(buf), " [%d, %d, %d, %d, %d, %d, %d, %d, %d, %d, %d, %d, %.6f]", s.kernel, s.macro_tile0,
             s.macro_tile1, s.depth_u, s.stages, s.wave_tile0, s.wave_tile1, s.split_k, s.raster, s.ctas,
             s.promote_k, s.tail_split, ms);
    lines[key] = buf;
    std::ofstream out(path, std::ios::trunc);
    if (!out) return fail(TL_ERR_INVALID_ARG, std::string("cannot write ") + path);
    out << "{\n";
    size_t i = 0;
    for (auto& kv : lines) {
        out << "\"" << kv.first << "\":" << kv.second << (++i < lines.size() ? ",\n" : "\n");
    }
    out << "}\n";
    return TL_SUCCESS;
}

}  // namespace

// Validation and launch description of a tcgen05 GEMM for a caller that supplies the scratch
// itself (tl_gemm_noalloc).  Allocates nothing: it only checks the problem and the solution and
// reports how much split-k workspace (bytes) and how many tile counters the launch needs.
tl_status plan_tc_noalloc(int device, int sm_count, size_t smem_optin, const tl_gemm_problem* prob,
                          const tl_gemm_solution* sol, void* D, const void* C, const void* A, const void* B,
                          TcLaunch* L, size_t* ws_bytes, size_t* counter_count)
{
    tl_status st = validate(prob);
    if (st != TL_SUCCESS) return st;
    // NN problems run as their transposed view where tl_gemm runs them so (same sums, same results)
    tl_gemm_solution s;
    bool tview = false;
    {
        tl_handle probe;           // host-side device description only
        probe.sm_count = sm_count;
        probe.smem_optin = smem_optin;
        if (sol) {
            s = *sol;
            if (s.kernel == TL_KERNEL_AUTO) s.kernel = TL_KERNEL_TCGEN05;
            tview = tc_nn_view(*prob, TL_KERNEL_TCGEN05) && view_solution_ok(s);
        } else {
            tc_heuristic_viewed(&probe, *prob, TL_KERNEL_TCGEN05, true, &s, &tview);
        }
    }
    const tl_gemm_problem view = tview ? nn_view(*prob) : *prob;
    if (tview) std::swap(A, B);
    const tl_gemm_problem& p = view;
    if (p.kernel != TL_KERNEL_AUTO && p.kernel != TL_KERNEL_TCGEN05)
        return fail(TL_ERR_UNSUPPORTED, "tl_gemm_noalloc runs the tcgen05 kernel only");
    if (p.dtype_a != TL_DTYPE_FP16 && p.dtype_a != TL_DTYPE_BF16 && p.dtype_a != TL_DTYPE_FP8_E4M3)
        return fail(TL_ERR_UNSUPPORTED, "tl_gemm_noalloc takes fp16, bf16 or fp8 operands");
    if ((p.m && p.n) && !D) return fail(TL_ERR_INVALID_ARG, "D is NULL");
    if (p.beta != 0.0f && !C && p.m && p.n) return fail(TL_ERR_INVALID_ARG, "C is NULL with beta != 0");
    if (p.k > 0 && p.m > 0 && p.n > 0 && (!A || !B)) return fail(TL_ERR_INVALID_ARG, "A or B is NULL");
    std::string why;
    if (p.m > 0 && p.n > 0 && p.k > 0 && !tma_ok(p, A, B, &why)) return fail(TL_ERR_UNSUPPORTED, "tcgen05 kernel: " + why);
    tl_handle dev;                 // host-side device description only; holds no device memory
    dev.sm_count = sm_count;
    dev.smem_optin = smem_optin;
    if (sol && s.kernel != TL_KERNEL_TCGEN05) return fail(TL_ERR_UNSUPPORTED, "tl_gemm_noalloc: solution must be TCGEN05");
    if (s.macro_tile1 == 4 * kTcTileN && p.m > 0 && p.n > 0 && p.k > 0 && !multicast_ok(A, B, device)) {
        if (sol) return multicast_refused();
        drop_cluster4(&dev, &s);
    }
    if ((st = check_tc_solution(&dev, p, s)) != TL_SUCCESS) return st;
    const int cgp = s.macro_tile1 / kTcTileN;
    const int64_t tiles = ((p.n + kTcTileN * cgp - 1) / (kTcTileN * cgp)) * cgp *
                          ((p.m + s.macro_tile0 - 1) / s.macro_tile0) * p.batch;
    *ws_bytes = (s.split_k > 1) ? static_cast<size_t>(tiles) * s.split_k * kTcTileN * s.macro_tile0 * sizeof(float) : 0;
    *counter_count = (s.split_k > 1) ? static_cast<size_t>(tiles) : 0;
    memset(L, 0, sizeof(*L));
    L->in_dtype = p.dtype_a;
    L->out_dtype = p.dtype_d;
    L->out_trunc = p.out_rounding;
    L->pieces = 1;
    L->opM[0] = {A, p.m, p.lda, p.stride_a, m_mn_major(p) ? 1 : 0};
    L->opN[0] = {B, p.n, p.ldb, p.stride_b, n_mn_major(p) ? 1 : 0};
    L->M = p.m; L->N = p.n; L->K = p.k; L->batch = p.batch;
    L->D = D; L->C = (p.beta != 0.0f) ? C : nullptr;
    L->ldd = p.ldd; L->ldc = p.ldc; L->stride_d = p.stride_d; L->stride_c = p.stride_c;
    L->alpha = p.alpha * scale_of(p.scale_a) * scale_of(p.scale_b);
    L->beta = p.beta;
    L->bm = s.macro_tile0;
    L->stages = s.stages;
    L->split_k = s.split_k;
    L->raster = s.raster;
    L->ctas = s.ctas;
    L->promote_k = s.promote_k;
    L->cg = cgp;
    L->tail_split = 1;     // the static scratch is sized for explicit split-k only
    L->debug_flags = s.debug_flags;
    L->epi_on = p.dtype_d == TL_DTYPE_FP8_E4M3 ? 1 : 0;     // fp8 outputs come out of the epilogue kernels
    L->epi_dscale = 1.0f;
    L->sm_count = sm_count;
    L->out_t = tview ? 1 : 0;
    return TL_SUCCESS;
}

}  // namespace tl

using namespace tl;

// =====================================================================================================
// C ABI
// =====================================================================================================
extern "C" {

TL_API const char* tl_last_error_string(void) { return g_last_error.c_str(); }

TL_API const char* tl_status_string(tl_status st)
{
    switch (st) {
    case TL_SUCCESS: return "TL_SUCCESS";
    case TL_WARN: return "TL_WARN";
    case TL_ERR: return "TL_ERR";
    case TL_FATAL: return "TL_FATAL";
    case TL_ERR_INVALID_ARG: return "TL_ERR_INVALID_ARG";
    case TL_ERR_UNSUPPORTED: return "TL_ERR_UNSUPPORTED";
    case TL_ERR_TIMEOUT: return "TL_ERR_TIMEOUT";
    case TL_ERR_CUDA: return "TL_ERR_CUDA";
    case TL_ERR_ALLOC: return "TL_ERR_ALLOC";
    default: return "TL_UNKNOWN";
    }
}

TL_API int tl_version(void) { return 10000; }

namespace {
tl_status host_only_refused()
{
    return fail(TL_ERR_INVALID_ARG, "planning handle (tl_init_host): it cannot launch, allocate or time work");
}
}  // namespace

TL_API tl_status tl_init(tl_handle** handle)
{
    if (!handle) return fail(TL_ERR_INVALID_ARG, "handle out-pointer is NULL");
    *handle = nullptr;
    tl_handle* h = new (std::nothrow) tl_handle();
    if (!h) return fail(TL_ERR_ALLOC, "handle allocation failed");
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaGetDevice"); }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, h->device);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaGetDeviceProperties"); }
    h->sm_count = prop.multiProcessorCount;
    h->cc_major = prop.major;
    h->cc_minor = prop.minor;
    h->smem_optin = prop.sharedMemPerBlockOptin;
    snprintf(h->name, sizeof(h->name), "%s", prop.name);
    if (const char* t = getenv("TL_WAIT_TIMEOUT_MS")) {
        long v = strtol(t, nullptr, 10);
        if (v > 0) h->timeout_ns = static_cast<uint64_t>(v) * 1000000ull;
    }
    if ((e = cudaMalloc(&h->d_err, 256)) != cudaSuccess) { delete h; return cuda_fail(e, "cudaMalloc(err)"); }
    h->d_norms = reinterpret_cast<double*>(reinterpret_cast<char*>(h->d_err) + 64);
    h->d_amax = reinterpret_cast<float*>(reinterpret_cast<char*>(h->d_err) + 128);
    if ((e = cudaMemset(h->d_err, 0, 256)) != cudaSuccess) { cudaFree(h->d_err); delete h; return cuda_fail(e, "cudaMemset"); }
    // the tuned-solution database of this device, when TL_SOLUTIONS names one (a missing file is no error)
    if (const char* path = getenv("TL_SOLUTIONS")) {
        std::ifstream probe(path);
        if (probe) tl_load_solutions(h, path, nullptr);
    }
    *handle = h;
    return TL_SUCCESS;
}

TL_API tl_status tl_init_host(int sm_count, size_t smem_optin, int clusters4, tl_handle** handle)
{
    if (!handle) return fail(TL_ERR_INVALID_ARG, "handle out-pointer is NULL");
    *handle = nullptr;
    if (sm_count < 1 || sm_count > 4096) return fail(TL_ERR_INVALID_ARG, "sm_count out of range");
    if (smem_optin < 16 * 1024 || smem_optin > 1024 * 1024) return fail(TL_ERR_INVALID_ARG, "smem_optin out of range");
    if (clusters4 < 0 || clusters4 > sm_count / 4) return fail(TL_ERR_INVALID_ARG, "clusters4 out of range");
    tl_handle* h = new (std::nothrow) tl_handle();
    if (!h) return fail(TL_ERR_ALLOC, "handle allocation failed");
    h->device = -1;
    h->sm_count = sm_count;
    h->cc_major = 10;
    h->cc_minor = 3;
    h->smem_optin = smem_optin;
    h->host_only = true;
    h->host_clusters4 = clusters4;
    snprintf(h->name, sizeof(h->name), "host description (%d SMs)", sm_count);
    *handle = h;
    return TL_SUCCESS;
}

TL_API tl_status tl_destroy(tl_handle* h)
{
    if (!h) return TL_SUCCESS;
    if (h->host_only) {
        delete h;
        return TL_SUCCESS;
    }
    cudaDeviceSynchronize();
    if (h->ws) cudaFree(h->ws);
    if (h->counters) cudaFree(h->counters);
    for (void* r : h->retired) cudaFree(r);
    for (cudaEvent_t e : h->tev) cudaEventDestroy(e);
    if (h->d_err) cudaFree(h->d_err);
    delete h;
    return TL_SUCCESS;
}

TL_API tl_status tl_device_info(tl_handle* h, int* sm_count, int* cc_major, int* cc_minor, size_t* smem)
{
    if (!h) return fail(TL_ERR_INVALID_ARG, "handle is NULL");
    if (sm_count) *sm_count = h->sm_count;
    if (cc_major) *cc_major = h->cc_major;
    if (cc_minor) *cc_minor = h->cc_minor;
    if (smem) *smem = h->smem_optin;
    return TL_SUCCESS;
}

TL_API tl_status tl_problem_init(tl_gemm_problem* p, tl_dtype ab, tl_dtype cd, tl_op ta, tl_op tb, int64_t m,
                                 int64_t n, int64_t k)
{
    if (!p) return fail(TL_ERR_INVALID_ARG, "problem is NULL");
    memset(p, 0, sizeof(*p));
    p->dtype_a = p->dtype_b = ab;
    p->dtype_c = p->dtype_d = cd;
    p->trans_a = ta;
    p->trans_b = tb;
    p->m = m; p->n = n; p->k = k;
    p->batch = 1;
    p->lda = std::max<int64_t>(1, ta == TL_OP_N ? m : k);
    p->ldb = std::max<int64_t>(1, tb == TL_OP_N ? k : n);
    p->ldc = p->ldd = std::max<int64_t>(1, m);
    p->stride_a = p->lda * (ta == TL_OP_N ? k : m);
    p->stride_b = p->ldb * (tb == TL_OP_N ? n : k);
    p->stride_c = p->stride_d = p->ldd * n;
    p->alpha = 1.0f;
    p->beta = 0.0f;
    p->scale_a = p->scale_b = 1.0f;
    p->kernel = TL_KERNEL_AUTO;
    p->out_rounding = TL_ROUND_RNE;
    return TL_SUCCESS;
}

TL_API tl_status tl_default_solution(tl_handle* h, const tl_gemm_problem* p, tl_gemm_solution* s)
{
    if (!h || !s) return fail(TL_ERR_INVALID_ARG, "NULL argument");
    tl_status st = validate(p);
    if (st != TL_SUCCESS) return st;
    const int kernel = resolve_kernel(*p);
    bool view = false;
    if (kernel == TL_KERNEL_SIMT) simt_solution(s);
    else tc_heuristic_viewed(h, *p, kernel, true, s, &view);
    return TL_SUCCESS;
}

TL_API tl_status tl_check_solution(tl_handle* h, const tl_gemm_problem* p, const tl_gemm_solution* s)
{
    if (!h || !s) return fail(TL_ERR_INVALID_ARG, "NULL argument");
    tl_status st = validate(p);
    if (st != TL_SUCCESS) return st;
    if (s->kernel == TL_KERNEL_SIMT) {
        if (s->macro_tile0 != 128 || s->macro_tile1 != 128 || (s->depth_u && s->depth_u != 8) || s->split_k > 1)
            return fail(TL_ERR_UNSUPPORTED, "SIMT kernel supports macro tile 128x128, depth_u 8, split_k 1");
        return TL_SUCCESS;
    }
    if (s->kernel != TL_KERNEL_TCGEN05 && !is_split(s->kernel))
        return fail(TL_ERR_INVALID_ARG, "solution kernel must be resolved (SIMT, TCGEN05, BF16X3 or BF16X6)");
    if (is_split(s->kernel) && p->dtype_a != TL_DTYPE_FP32)
        return fail(TL_ERR_UNSUPPORTED, "bf16x3/bf16x6 need fp32 inputs");
    if (s->kernel == TL_KERNEL_TCGEN05 && p->dtype_a == TL_DTYPE_FP32)
        return fail(TL_ERR_UNSUPPORTED, "tcgen05 kernel needs fp16/bf16/fp8 inputs");
    return check_tc_solution(h, tc_nn_view(*p, s->kernel) && view_solution_ok(*s) ? nn_view(*p) : *p, *s);
}

TL_API tl_status tl_gemm(tl_handle* h, const tl_gemm_problem* p, const tl_gemm_solution* s, void* D, const void* C,
                         const void* A, const void* B, void* stream)
{
    if (h && h->host_only) return host_only_refused();
    if (!h) return fail(TL_ERR_INVALID_ARG, "handle is NULL");
    Prepared P;
    t_capturing = stream_capturing(S(stream));
    if (t_capturing) h->captured = true;
    tl_status st = prepare(h, p, s, D, C, A, B, &P);
    t_capturing = false;
    if (st != TL_SUCCESS) return st;
    return enqueue(h, P, S(stream));
}

// ---- Tensile-layout entry -------------------------------------------------------------------------
// Fields of the packed argument buffer (no alignment assumed).
static uint64_t karg_u64(const void* buf, size_t off)
{
    uint64_t v;
    memcpy(&v, static_cast<const char*>(buf) + off, sizeof(v));
    return v;
}
static uint32_t karg_u32(const void* buf, size_t off)
{
    uint32_t v;
    memcpy(&v, static_cast<const char*>(buf) + off, sizeof(v));
    return v;
}
static void* karg_ptr(const void* buf, size_t off)
{
    void* v;
    memcpy(&v, static_cast<const char*>(buf) + off, sizeof(v));
    return v;
}

// Last element touched by a TN operand or the output, +1 (elements): the extent to check against
// the buffer size the caller declared.
static uint64_t tn_extent(uint64_t rows, uint64_t cols, uint64_t ld, uint64_t batch, uint64_t batch_stride)
{
    if (rows == 0 || cols == 0 || batch == 0) return 0;
    return (batch - 1) * batch_stride + (cols - 1) * ld + rows;
}

TL_API tl_status tl_tensile_launch(tl_handle* h, const char* kernel_name, const void* kernarg, size_t kernarg_bytes,
                                   void* stream)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || !kernel_name || !kernarg) return fail(TL_ERR_INVALID_ARG, "NULL argument");
    if (kernarg_bytes < TL_TENSILE_KERNARG_BYTES)
        return fail(TL_ERR_INVALID_ARG, "Tensile argument buffer shorter than 148 bytes");
    const std::string name(kernel_name);
    const std::string prefix = "Cijk_Alik_Bljk_";
    if (name.compare(0, prefix.size(), prefix) != 0)
        return fail(TL_ERR_UNSUPPORTED, "Tensile kernel " + name + ": only Cijk_Alik_Bljk (TN) is provided");
    const std::string rest = name.substr(prefix.size());
    auto is = [&](const char* tag) {
        const size_t n = strlen(tag);
        return rest.compare(0, n, tag) == 0 && (rest.size() == n || rest[n] == '_');
    };
    tl_dtype dt;
    if (is("SB")) dt = TL_DTYPE_FP32;
    else if (is("HBH")) dt = TL_DTYPE_FP16;
    else if (is("BBH")) dt = TL_DTYPE_BF16;
    else return fail(TL_ERR_UNSUPPORTED, "Tensile kernel " + name + ": data types must be SB, HBH or BBH");

    const uint64_t size_c = karg_u64(kernarg, 0), size_a = karg_u64(kernarg, 8), size_b = karg_u64(kernarg, 16);
    void* D = karg_ptr(kernarg, 24);
    const void* C = karg_ptr(kernarg, 32);
    const void* A = karg_ptr(kernarg, 40);
    const void* B = karg_ptr(kernarg, 48);
    const uint32_t alpha_bits = karg_u32(kernarg, 56), beta_bits = karg_u32(kernarg, 60);
    uint32_t st[8];
    for (int i = 0; i < 8; ++i) st[i] = karg_u32(kernarg, 64 + 4 * i);   // D0 D1 C0 C1 A0 A1 B0 B1
    const uint32_t M = karg_u32(kernarg, 96), N = karg_u32(kernarg, 100), batch = karg_u32(kernarg, 104),
                   K = karg_u32(kernarg, 108);
    float alpha, beta;
    if (dt == TL_DTYPE_FP16) {
        // the HBH kernel takes alpha/beta as fp16 (converted in the kernel, src/gemmMfmaKernelWriter.h:1845-1854)
        __half_raw ra, rb;
        ra.x = static_cast<unsigned short>(alpha_bits & 0xFFFFu);
        rb.x = static_cast<unsigned short>(beta_bits & 0xFFFFu);
        alpha = __half2float(__half(ra));
        beta = __half2float(__half(rb));
    } else {
        memcpy(&alpha, &alpha_bits, 4);
        memcpy(&beta, &beta_bits, 4);
    }
    tl_gemm_problem p;
    tl_status st0 = tl_problem_init(&p, dt, dt, TL_OP_T, TL_OP_N, M, N, K);
    if (st0 != TL_SUCCESS) return st0;
    p.batch = batch;
    p.ldd = st[0]; p.stride_d = st[1];
    p.ldc = st[2]; p.stride_c = st[3];
    p.lda = st[4]; p.stride_a = st[5];
    p.ldb = st[6]; p.stride_b = st[7];
    p.alpha = alpha;
    p.beta = beta;
    if (dt == TL_DTYPE_BF16) p.out_rounding = TL_ROUND_TRUNCATE;   // the reference kernel's bf16 store
    // the declared buffer sizes bound every access
    if ((size_a && tn_extent(K, M, st[4], batch, st[5]) > size_a) ||
        (size_b && tn_extent(K, N, st[6], batch, st[7]) > size_b) ||
        (size_c && (tn_extent(M, N, st[0], batch, st[1]) > size_c ||
                    (beta != 0.0f && tn_extent(M, N, st[2], batch, st[3]) > size_c))))
        return fail(TL_ERR_INVALID_ARG, "Tensile arguments: strides and sizes exceed a declared buffer size");
    return tl_gemm(h, &p, nullptr, D, C, A, B, stream);
}

TL_API tl_status tl_gemm_ex(tl_handle* h, const tl_gemm_problem* p, const tl_epilogue* epi,
                            const tl_gemm_solution* s, void* D, const void* C, const void* A, const void* B, void* stream)
{
    if (h && h->host_only) return host_only_refused();
    if (!h) return fail(TL_ERR_INVALID_ARG, "handle is NULL");
    if (!epi) return tl_gemm(h, p, s, D, C, A, B, stream);
    if (epi->activation < TL_ACT_NONE || epi->activation > TL_ACT_SILU)
        return fail(TL_ERR_INVALID_ARG, "epilogue activation must be NONE, RELU, GELU or SILU");
    if (epi->bias && epi->bias_dtype != TL_DTYPE_FP32 && epi->bias_dtype != TL_DTYPE_FP16 &&
        epi->bias_dtype != TL_DTYPE_BF16)
        return fail(TL_ERR_INVALID_ARG, "epilogue bias must be fp32, fp16 or bf16");
    if (epi->bias && (reinterpret_cast<uintptr_t>(epi->bias) % dtype_bytes(epi->bias_dtype)))
        return fail(TL_ERR_INVALID_ARG, "epilogue bias is not aligned to its element size");
    if (epi->amax && (reinterpret_cast<uintptr_t>(epi->amax) & 3))
        return fail(TL_ERR_INVALID_ARG, "epilogue amax is not 4-byte aligned");
    if (!(epi->d_scale >= 0.0f) || std::isinf(epi->d_scale))
        return fail(TL_ERR_INVALID_ARG, "epilogue d_scale must be finite and >= 0 (0 is read as 1)");
    Prepared P;
    t_capturing = stream_capturing(S(stream));
    if (t_capturing) h->captured = true;
    tl_status st = prepare(h, p, s, D, C, A, B, &P, true);
    t_capturing = false;
    if (st != TL_SUCCESS) return st;
    if (P.kernel == TL_KERNEL_SIMT)
        return fail(TL_ERR_UNSUPPORTED, "a fused epilogue needs a tensor-core kernel (fp16/bf16/fp8 operands, or "
                                        "fp32 with BF16X3/BF16X6)");
    if (P.p.k == 0 || P.p.m == 0 || P.p.n == 0)
        return fail(TL_ERR_UNSUPPORTED, "a fused epilogue needs m, n, k > 0");
    P.epi = *epi;
    P.epi_on = epi->bias != nullptr || epi->activation != TL_ACT_NONE || epi->amax != nullptr ||
               (P.p.dtype_d == TL_DTYPE_FP8_E4M3 && epi->d_scale != 0.0f && epi->d_scale != 1.0f);
    return enqueue(h, P, S(stream));
}

TL_API tl_status tl_tune(tl_handle* h, const tl_gemm_problem* p, void* D, const void* C, const void* A,
                         const void* B, int max_candidates, int reps, const char* cache_path, tl_gemm_solution* best,
                         float* best_ms)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || !best) return fail(TL_ERR_INVALID_ARG, "NULL argument");
    tl_status st = validate(p);
    if (st != TL_SUCCESS) return st;
    const int kernel = resolve_kernel(*p);
    std::vector<tl_gemm_solution> cands;
    if (kernel == TL_KERNEL_SIMT) {
        tl_gemm_solution s;
        simt_solution(&s);
        cands.push_back(s);
    } else {
        cands = tc_candidates(h, tc_nn_view(*p, kernel) ? nn_view(*p) : *p, kernel);
    }
    // the multicast variant only where A and B are this GPU's memory
    if (!multicast_ok(A, B, h->device))
        cands.erase(std::remove_if(cands.begin(), cands.end(),
                                   [](const tl_gemm_solution& c) { return c.macro_tile1 == 4 * kTcTileN; }),
                    cands.end());
    if (cands.empty()) return fail(TL_ERR_UNSUPPORTED, "no legal candidate solution");
    if (max_candidates <= 0) max_candidates = 16;
    if (reps <= 0) reps = 10;
    if (static_cast<int>(cands.size()) > max_candidates) cands.resize(max_candidates);
    if ((st = bind_thread(h)) != TL_SUCCESS) return st;
    // in place (D == C, beta != 0): every timed launch would fold beta*C into C again, so the
    // candidates read C where it is and write a scratch output of D's extent instead
    void* Dt = D;
    void* scratch = nullptr;
    if (D != nullptr && D == C && p->beta != 0.0f && p->m > 0 && p->n > 0) {
        const size_t bytes = static_cast<size_t>(operand_span(p->ldd, p->n, p->batch, p->stride_d, p->m)) *
                             dtype_bytes(p->dtype_d);
        if (cudaMalloc(&scratch, bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(TL_ERR_ALLOC, "tuner scratch output allocation failed");
        }
        Dt = scratch;
    }
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        if (scratch) cudaFree(scratch);
        return fail(TL_ERR_CUDA, "stream create");
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_t = 1e30f;
    tl_gemm_solution best_s = cands[0];
    bool any = false;
    std::string dropped;
    // a candidate counts only if its launches finished without a device error: a bounded wait that
    // ran out returns early and would look fastest
    auto device_clean = [&](const tl_gemm_solution& c) {
        int v = 0;
        if (cudaStreamSynchronize(s) != cudaSuccess || cudaMemcpy(&v, h->d_err, sizeof(int), cudaMemcpyDeviceToHost) !=
                                                           cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (v != 0) {
            cudaMemset(h->d_err, 0, sizeof(int));
            char buf[160];
            snprintf(buf, sizeof(buf), " [mt %dx%d split %d: device wait timed out, mask 0x%x]", c.macro_tile0,
                     c.macro_tile1, c.split_k, v);
            dropped += buf;
            return false;
        }
        return true;
    };
    for (const auto& c : cands) {
        Prepared P;
        if (prepare(h, p, &c, Dt, C, A, B, &P) != TL_SUCCESS) continue;
        if (enqueue(h, P, s) != TL_SUCCESS) continue;          // warm-up
        if (!device_clean(c)) continue;
        cudaEventRecord(e0, s);
        bool ok = true;
        for (int r = 0; r < reps && ok; ++r) ok = enqueue(h, P, s) == TL_SUCCESS;
        cudaEventRecord(e1, s);
        if (!ok || cudaEventSynchronize(e1) != cudaSuccess) { cudaGetLastError(); continue; }
        if (!device_clean(c)) continue;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= reps;
        any = true;
        if (ms < best_t) { best_t = ms; best_s = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    if (scratch) cudaFree(scratch);
    if (!any) return fail(TL_ERR_UNSUPPORTED, "every candidate failed: " + g_last_error + dropped);
    *best = best_s;
    if (best_ms) *best_ms = best_t;
    const std::string key = problem_key(h, *p);
    {
        std::lock_guard<std::mutex> g(h->mu);
        h->tuned[key] = best_s;
    }
    if (cache_path) return save_cache(cache_path, key, best_s, best_t);
    return TL_SUCCESS;
}

TL_API tl_status tl_load_solutions(tl_handle* h, const char* path, int* loaded)
{
    if (!h || !path) return fail(TL_ERR_INVALID_ARG, "NULL argument");
    std::ifstream in(path);
    if (!in) return fail(TL_ERR_INVALID_ARG, std::string("cannot read ") + path);
    std::string line;
    int n = 0;
    const std::string prefix = std::string(h->name) + "|sm" + std::to_string(h->cc_major) + std::to_string(h->cc_minor) + "|";
    while (std::getline(in, line)) {
        size_t q0 = line.find('"');
        size_t q1 = line.find("\":", q0 + 1);
        size_t b0 = line.find('[', q1 == std::string::npos ? 0 : q1);
        if (q0 == std::string::npos || q1 == std::string::npos || b0 == std::string::npos) continue;
        std::string key = line.substr(q0 + 1, q1 - q0 - 1);
        if (key.compare(0, prefix.size(), prefix) != 0) continue;   // other device
        tl_gemm_solution s;
        memset(&s, 0, sizeof(s));
        float ms = 0;
        if (sscanf(line.c_str() + b0, "[%d, %d, %d, %d, %d, %d, %d, %d, %d, %d, %d, %d, %f", &s.kernel,
                   &s.macro_tile0, &s.macro_tile1, &s.depth_u, &s.stages, &s.wave_tile0, &s.wave_tile1, &s.split_k,
                   &s.raster, &s.ctas, &s.promote_k, &s.tail_split, &ms) == 13) {
            std::lock_guard<std::mutex> g(h->mu);
            h->tuned[key] = s;
            ++n;
        }
    }
    if (loaded) *loaded = n;
    return TL_SUCCESS;
}

// ---- grouped ---------------------------------------------------------------------------------------
TL_API tl_status tl_grouped_plan_create(tl_handle* h, const tl_gemm_problem* probs, int count, void* const* D,
                                        const void* const* C, const void* const* A, const void* const* B,
                                        const tl_gemm_solution* sol, tl_grouped_plan** plan)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || !probs || !plan || count < 1 || !D || !A || !B) return fail(TL_ERR_INVALID_ARG, "NULL argument or count < 1");
    *plan = nullptr;
    const tl_gemm_problem& p0 = probs[0];
    tl_status st = bind_thread(h);
    if (st != TL_SUCCESS) return st;
    for (int i = 0; i < count; ++i) {
        const tl_gemm_problem& p = probs[i];
        if ((st = validate(&p)) != TL_SUCCESS) return fail(st, "problem " + std::to_string(i) + ": " + g_last_error);
        if (p.dtype_a != p0.dtype_a || p.dtype_d != p0.dtype_d || p.trans_a != p0.trans_a || p.trans_b != p0.trans_b ||
            p.out_rounding != p0.out_rounding)
            return fail(TL_ERR_UNSUPPORTED, "grouped problems must share dtypes, trans flags and rounding");
        if (p.batch != 1) return fail(TL_ERR_UNSUPPORTED, "grouped problems must have batch == 1");
        if (p.dtype_d == TL_DTYPE_FP8_E4M3) return fail(TL_ERR_UNSUPPORTED, "grouped GEMM writes no fp8 output");
        if (p.k == 0) return fail(TL_ERR_UNSUPPORTED, "grouped problems need k > 0");
        if (p.beta != 0.0f && (!C || !C[i])) return fail(TL_ERR_INVALID_ARG, "C missing with beta != 0");
        std::string why;
        tl_gemm_problem q = p;
        q.kernel = TL_KERNEL_TCGEN05;
        if (!tma_ok(q, A[i], B[i], &why)) return fail(TL_ERR_UNSUPPORTED, "problem " + std::to_string(i) + ": " + why);
    }
    if (p0.dtype_a != TL_DTYPE_FP16 && p0.dtype_a != TL_DTYPE_BF16 && p0.dtype_a != TL_DTYPE_FP8_E4M3)
        return fail(TL_ERR_UNSUPPORTED, "grouped GEMM takes fp16/bf16/fp8 operands");
    tl_gemm_solution s;
    if (sol) {
        s = *sol;
    } else {
        // heuristic for a group: the tile that suits the median problem
        std::vector<int64_t> ms;
        for (int i = 0; i < count; ++i) ms.push_back(probs[i].m);
        std::nth_element(ms.begin(), ms.begin() + count / 2, ms.end());
        tl_gemm_problem med = p0;
        med.m = ms[count / 2];
        med.kernel = TL_KERNEL_TCGEN05;
        tc_heuristic(h, med, TL_KERNEL_TCGEN05, &s);
        // a CTA pair per 256 x 256 tile (half the m-side operand per SM) where every problem allows it
        s.macro_tile0 = 256;
        s.macro_tile1 = 2 * kTcTileN;
        s.stages = std::min(6, max_stages(s.macro_tile0 / 2, h->smem_optin));
        s.split_k = 1;
        s.raster = 0;
        s.tail_split = 0;
        for (int i = 0; i < count; ++i)
            if (check_tc_solution(h, probs[i], s) != TL_SUCCESS) {
                s.macro_tile1 = kTcTileN;
                s.stages = max_stages(s.macro_tile0, h->smem_optin);
                break;
            }
    }
    s.kernel = TL_KERNEL_TCGEN05;
    if (s.split_k == 0) s.split_k = 1;
    if (s.split_k != 1) return fail(TL_ERR_UNSUPPORTED, "grouped GEMM does not split k");
    if (s.macro_tile1 == 4 * kTcTileN) {
        // the multicast variant only where every problem's A and B are this GPU's memory
        bool local = true;
        for (int i = 0; i < count && local; ++i) local = multicast_ok(A[i], B[i], h->device);
        if (!local) {
            if (sol) return multicast_refused();
            drop_cluster4(h, &s);
        }
    }
    for (int i = 0; i < count; ++i)
        if ((st = check_tc_solution(h, probs[i], s)) != TL_SUCCESS) return st;

    std::vector<TcGroupEntry> host(count);
    std::vector<int64_t> prefix(count + 1, 0);
    const int kb_elems = tl::kTcRowBytes / (p0.dtype_a == TL_DTYPE_FP8_E4M3 ? 1 : 2);
    double flops = 0;
    for (int i = 0; i < count; ++i) {
        const tl_gemm_problem& p = probs[i];
        TcGroupEntry& e = host[i];
        memset(&e, 0, sizeof(e));
        TcOperand opN{B[i], p.n, p.ldb, p.stride_b, n_mn_major(p) ? 1 : 0};
        TcOperand opM{A[i], p.m, p.lda, p.stride_a, m_mn_major(p) ? 1 : 0};
        if (p.m > 0 && p.n > 0) {
            if ((st = tc_encode_operand(&e.tmN, p.dtype_a, opN, p.k, 1, kTcTileN)) != TL_SUCCESS) return st;
            if ((st = tc_encode_operand(&e.tmM, p.dtype_a, opM, p.k, 1, s.macro_tile0 * kTcTileN / s.macro_tile1)) !=
                TL_SUCCESS)
                return st;
        }
        e.D = D[i];
        e.C = (p.beta != 0.0f && C) ? C[i] : nullptr;
        e.ldd = p.ldd;
        e.ldc = p.ldc;
        e.M = static_cast<int32_t>(p.m);
        e.N = static_cast<int32_t>(p.n);
        e.K = static_cast<int32_t>(p.k);
        e.tiles_m = static_cast<int32_t>((p.m + s.macro_tile0 - 1) / s.macro_tile0);
        e.tiles_n = static_cast<int32_t>((p.n + s.macro_tile1 - 1) / s.macro_tile1);
        e.alpha = p.alpha * scale_of(p.scale_a) * scale_of(p.scale_b);
        e.beta = p.beta;
        e.tma_store = (p.m > 0 && p.n > 0 &&
                       tc_encode_output(&e.tmD, p.dtype_d, D[i], p.m, p.n, p.ldd, 1, p.stride_d)) ? 1 : 0;
        prefix[i + 1] = prefix[i] + static_cast<int64_t>(e.tiles_m) * e.tiles_n;
        flops += 2.0 * static_cast<double>(p.m) * p.n * p.k;
    }
    // The unit table: work unit w -> (problem, tile row along n, tile column along m, k-blocks), in
    // problem order, tiles of a problem n-major.  The kernel reads one 16-byte entry per tile
    // (loaded a tile ahead) instead of searching the per-problem tile prefix.
    const int64_t total_units = prefix[count];
    if (total_units > INT32_MAX) return fail(TL_ERR_UNSUPPORTED, "grouped plan has too many tiles");
    std::vector<int4> units(static_cast<size_t>(total_units));
    // problems in order of decreasing k: the tiles running side by side then take about as long,
    // so the workers stay in step (tiles sharing operand rows read them while they are in L2) and
    // the launch ends with its shortest tiles
    std::vector<int> order(count);
    for (int i = 0; i < count; ++i) order[i] = i;
    if (group_order_by_k())
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return host[a].K > host[b].K; });
    for (int oi = 0, w = 0; oi < count; ++oi) {
        const int i = order[oi];
        const TcGroupEntry& e = host[i];
        const int nkb = static_cast<int>((e.K + kb_elems - 1) / kb_elems);
        for (int in = 0; in < e.tiles_n; ++in)
            for (int jm = 0; jm < e.tiles_m; ++jm) units[w++] = make_int4(i, in, jm, nkb);
    }
    tl_grouped_plan* pl = new (std::nothrow) tl_grouped_plan();
    if (!pl) return fail(TL_ERR_ALLOC, "plan allocation failed");
    pl->h = h;
    cudaError_t e;
    if ((e = cudaMalloc(&pl->d_entries, sizeof(TcGroupEntry) * count)) != cudaSuccess ||
        (total_units > 0 && (e = cudaMalloc(&pl->d_units, sizeof(int4) * units.size())) != cudaSuccess)) {
        tl_grouped_plan_destroy(pl);
        return cuda_fail(e, "cudaMalloc(plan)");
    }
    if ((e = cudaMemcpy(pl->d_entries, host.data(), sizeof(TcGroupEntry) * count, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (total_units > 0 &&
         (e = cudaMemcpy(pl->d_units, units.data(), sizeof(int4) * units.size(), cudaMemcpyHostToDevice)) != cudaSuccess)) {
        tl_grouped_plan_destroy(pl);
        return cuda_fail(e, "cudaMemcpy(plan)");
    }
    TcGroupLaunch& G = pl->launch;
    G.in_dtype = p0.dtype_a;
    G.out_dtype = p0.dtype_d;
    G.out_trunc = p0.out_rounding;
    G.n_mn_major = n_mn_major(p0) ? 1 : 0;
    G.m_mn_major = m_mn_major(p0) ? 1 : 0;
    G.d_entries = pl->d_entries;
    G.d_units = pl->d_units;
    G.count = count;
    G.total_tiles = prefix[count];
    G.bm = s.macro_tile0;
    G.stages = s.stages;
    G.ctas = s.ctas;
    G.cg = s.macro_tile1 / kTcTileN;
    G.err = h->d_err;
    G.timeout_ns = h->timeout_ns;
    G.sm_count = h->sm_count;
    pl->sol = s;
    pl->flops = flops;
    *plan = pl;
    return TL_SUCCESS;
}

TL_API tl_status tl_grouped_plan_launch(tl_grouped_plan* pl, void* stream)
{
    if (!pl) return fail(TL_ERR_INVALID_ARG, "plan is NULL");
    if (pl->launch.total_tiles == 0) return TL_SUCCESS;
    const bool timed = timing_begin(pl->h, S(stream));
    const tl_status st = tc_grouped_launch(pl->launch, S(stream), &pl->h->launches);
    timing_end(pl->h, S(stream), timed, st);
    return st;
}

TL_API tl_status tl_grouped_plan_destroy(tl_grouped_plan* pl)
{
    if (!pl) return TL_SUCCESS;
    if (pl->d_entries || pl->d_units) cudaDeviceSynchronize();
    if (pl->d_entries) cudaFree(pl->d_entries);
    if (pl->d_units) cudaFree(pl->d_units);
    delete pl;
    return TL_SUCCESS;
}

TL_API tl_status tl_grouped_plan_info(const tl_grouped_plan* pl, double* flops, int64_t* tiles, tl_gemm_solution* s)
{
    if (!pl) return fail(TL_ERR_INVALID_ARG, "plan is NULL");
    if (flops) *flops = pl->flops;
    if (tiles) *tiles = pl->launch.total_tiles;
    if (s) *s = pl->sol;
    return TL_SUCCESS;
}

TL_API tl_status tl_gemm_grouped(tl_handle* h, const tl_gemm_problem* probs, int count, void* const* D,
                                 const void* const* C, const void* const* A, const void* const* B, void* stream)
{
    if (h && h->host_only) return host_only_refused();
    tl_grouped_plan* pl = nullptr;
    tl_status st = tl_grouped_plan_create(h, probs, count, D, C, A, B, nullptr, &pl);
    if (st != TL_SUCCESS) return st;
    st = tl_grouped_plan_launch(pl, stream);
    if (st == TL_SUCCESS) {
        cudaError_t e = cudaStreamSynchronize(S(stream));
        if (e != cudaSuccess) st = cuda_fail(e, "cudaStreamSynchronize(grouped)");
    }
    tl_grouped_plan_destroy(pl);
    return st;
}

TL_API tl_status tl_tune_grouped(tl_handle* h, const tl_gemm_problem* probs, int count, void* const* D,
                                 const void* const* C, const void* const* A, const void* const* B, int reps,
                                 tl_gemm_solution* best, float* best_ms)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || !best || count < 1) return fail(TL_ERR_INVALID_ARG, "NULL argument");
    if (reps <= 0) reps = 5;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return fail(TL_ERR_CUDA, "stream create");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_t = 1e30f;
    bool any = false;
    for (int cg : {1, 2, 4})
    for (int bm : {64, 128, 192, 256}) {
        for (int stages : {3, 4, 6, 8}) {
            if (cg == 4 && !cluster4_enabled()) continue;
            tl_gemm_solution c;
            memset(&c, 0, sizeof(c));
            c.kernel = TL_KERNEL_TCGEN05;
            c.macro_tile0 = bm;
            c.macro_tile1 = kTcTileN * cg;
            c.stages = std::min(stages, max_stages(bm / (cg >= 2 ? 2 : 1), h->smem_optin));
            c.split_k = 1;
            if (stages > c.stages) continue;
            tl_grouped_plan* pl = nullptr;
            if (tl_grouped_plan_create(h, probs, count, D, C, A, B, &c, &pl) != TL_SUCCESS) continue;
            bool ok = tl_grouped_plan_launch(pl, s) == TL_SUCCESS && cudaStreamSynchronize(s) == cudaSuccess;
            if (ok) {
                cudaEventRecord(e0, s);
                for (int r = 0; r < reps && ok; ++r) ok = tl_grouped_plan_launch(pl, s) == TL_SUCCESS;
                cudaEventRecord(e1, s);
                ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
            }
            if (ok) {
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= reps;
                any = true;
                if (ms < best_t) { best_t = ms; *best = pl->sol; }
            }
            tl_grouped_plan_destroy(pl);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    if (!any) return fail(TL_ERR_UNSUPPORTED, "every grouped candidate failed: " + g_last_error);
    if (best_ms) *best_ms = best_t;
    return TL_SUCCESS;
}

// ---- graphs ----------------------------------------------------------------------------------------
static tl_status end_capture(cudaStream_t s, tl_status inner, tl_graph** out)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (inner != TL_SUCCESS) {
        if (g) cudaGraphDestroy(g);
        return inner;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    tl_graph* gr = new (std::nothrow) tl_graph();
    if (!gr) { cudaGraphDestroy(g); return fail(TL_ERR_ALLOC, "graph allocation failed"); }
    gr->graph = g;
    e = cudaGraphInstantiate(&gr->exec, g, 0);
    if (e != cudaSuccess) { cudaGraphDestroy(g); delete gr; return cuda_fail(e, "cudaGraphInstantiate"); }
    *out = gr;
    return TL_SUCCESS;
}

TL_API tl_status tl_graph_capture_grouped(tl_grouped_plan* pl, void* stream, tl_graph** out)
{
    if (!pl || !out || !stream) return fail(TL_ERR_INVALID_ARG, "NULL argument (capture needs a non-default stream)");
    cudaStream_t s = S(stream);
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    tl_status st = tl_grouped_plan_launch(pl, stream);
    return end_capture(s, st, out);
}

TL_API tl_status tl_graph_capture_gemm(tl_handle* h, const tl_gemm_problem* p, const tl_gemm_solution* sol, void* D,
                                       const void* C, const void* A, const void* B, void* stream, tl_graph** out)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || !out || !stream) return fail(TL_ERR_INVALID_ARG, "NULL argument (capture needs a non-default stream)");
    Prepared P;
    tl_status st = prepare(h, p, sol, D, C, A, B, &P);   // allocations happen before capture
    if (st != TL_SUCCESS) return st;
    h->captured = true;
    cudaStream_t s = S(stream);
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    st = enqueue(h, P, s);
    return end_capture(s, st, out);
}

TL_API tl_status tl_graph_launch(tl_graph* g, void* stream)
{
    if (!g) return fail(TL_ERR_INVALID_ARG, "graph is NULL");
    TL_CUDA_TRY(cudaGraphLaunch(g->exec, S(stream)));
    return TL_SUCCESS;
}

TL_API tl_status tl_graph_destroy(tl_graph* g)
{
    if (!g) return TL_SUCCESS;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return TL_SUCCESS;
}

// ---- fp8 / split -------------------------------------------------------------------------------------
TL_API tl_status tl_quantize_fp8(tl_handle* h, tl_dtype src_dtype, const void* src, int64_t n, void* dst,
                                 float* scale_out, float* amax_out, void* stream)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || (!src && n) || (!dst && n) || n < 0) return fail(TL_ERR_INVALID_ARG, "bad argument");
    if (src_dtype != TL_DTYPE_FP32 && src_dtype != TL_DTYPE_FP16 && src_dtype != TL_DTYPE_BF16)
        return fail(TL_ERR_UNSUPPORTED, "quantize: source must be fp32, fp16 or bf16");
    float* amax = amax_out ? amax_out : h->d_amax;
    tl_status st = aux_amax(src_dtype, src, n, amax, S(stream), &h->launches);
    if (st != TL_SUCCESS) return st;
    return aux_quant_e4m3(src_dtype, src, n, amax, static_cast<uint8_t*>(dst), scale_out, S(stream), &h->launches);
}

TL_API tl_status tl_split_bf16x2(tl_handle* h, const float* src, int64_t n, void* hi, void* lo, void* stream)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || n < 0 || (n && (!src || !hi || !lo))) return fail(TL_ERR_INVALID_ARG, "bad argument");
    return aux_split_bf16(src, n, 1, n, 1, n, static_cast<uint16_t*>(hi), static_cast<uint16_t*>(lo), nullptr,
                          S(stream), &h->launches);
}

// ---- verification ------------------------------------------------------------------------------------
TL_API tl_status tl_error_norms(tl_handle* h, tl_dtype dtype_d, const void* D, int64_t ldd, const double* R,
                                const double* W, int64_t ldr, int64_t m, int64_t n, double out[3], void* stream)
{
    if (h && h->host_only) return host_only_refused();
    if (!h || !out || m < 0 || n < 0 || ldd < m || ldr < m) return fail(TL_ERR_INVALID_ARG, "bad argument");
    if (dtype_bytes(dtype_d) == 0) return fail(TL_ERR_INVALID_ARG, "bad dtype");
    tl_status st = aux_error_norms(dtype_d, D, ldd, R, W, ldr, m, n, h->d_norms, S(stream), &h->launches);
    if (st != TL_SUCCESS) return st;
    TL_CUDA_TRY(cudaMemcpyAsync(out, h->d_norms, 3 * sizeof(double), cudaMemcpyDeviceToHost, S(stream)));
    TL_CUDA_TRY(cudaStreamSynchronize(S(stream)));
    return TL_SUCCESS;
}

// ---- buffers -------------------------------------------------------------------------------------
TL_API tl_status tl_malloc(void** p, size_t bytes)
{
    if (!p) return fail(TL_ERR_INVALID_ARG, "NULL out-pointer");
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 1);
    if (e != cudaSuccess) { *p = nullptr; return fail(TL_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e)); }
    return TL_SUCCESS;
}
TL_API tl_status tl_free(void* p) { TL_CUDA_TRY(cudaFree(p)); return TL_SUCCESS; }
TL_API tl_status tl_host_malloc(void** p, size_t bytes)
{
    if (!p) return fail(TL_ERR_INVALID_ARG, "NULL out-pointer");
    cudaError_t e = cudaMallocHost(p, bytes ? bytes : 1);
    if (e != cudaSuccess) { *p = nullptr; return fail(TL_ERR_ALLOC, std::string("cudaMallocHost: ") + cudaGetErrorString(e)); }
    return TL_SUCCESS;
}
TL_API tl_status tl_host_free(void* p) { TL_CUDA_TRY(cudaFreeHost(p)); return TL_SUCCESS; }
TL_API tl_status tl_memcpy_h2d(void* d, const void* s, size_t b, void* st)
{ TL_CUDA_TRY(cudaMemcpyAsync(d, s, b, cudaMemcpyHostToDevice, S(st))); return TL_SUCCESS; }
TL_API tl_status tl_memcpy_d2h(void* d, const void* s, size_t b, void* st)
{ TL_CUDA_TRY(cudaMemcpyAsync(d, s, b, cudaMemcpyDeviceToHost, S(st))); return TL_SUCCESS; }
TL_API tl_status tl_memcpy_d2d(void* d, const void* s, size_t b, void* st)
{ TL_CUDA_TRY(cudaMemcpyAsync(d, s, b, cudaMemcpyDeviceToDevice, S(st))); return TL_SUCCESS; }
TL_API tl_status tl_memset(void* d, int v, size_t b, void* st)
{ TL_CUDA_TRY(cudaMemsetAsync(d, v, b, S(st))); return TL_SUCCESS; }
TL_API tl_status tl_stream_create(void** s)
{
    if (!s) return fail(TL_ERR_INVALID_ARG, "NULL out-pointer");
    cudaStream_t st;
    TL_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    *s = st;
    return TL_SUCCESS;
}
TL_API tl_status tl_stream_destroy(void* s) { TL_CUDA_TRY(cudaStreamDestroy(S(s))); return TL_SUCCESS; }
TL_API tl_status tl_stream_synchronize(void* s) { TL_CUDA_TRY(cudaStreamSynchronize(S(s))); return TL_SUCCESS; }

TL_API tl_status tl_fill_pattern(tl_dtype dtype, void* dst, int64_t count, float code, void* stream)
{
    if (dtype_bytes(dtype) == 0 || count < 0 || (count && !dst)) return fail(TL_ERR_INVALID_ARG, "bad argument");
    if (code == 2.2f || code == -2.2f)
        return fail(TL_ERR_UNSUPPORTED, "patterns 2.2/-2.2 depend on the buffer shape; fill them on the host");
    return aux_fill_pattern(dtype, dst, count, code, S(stream), nullptr);
}

// Host converters (IEEE round-to-nearest-even unless TRUNCATE is asked for bf16).
static uint16_t host_f32_to_f16(float f)
{
    uint32_t x;
    memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t e = (x >> 23) & 0xffu;
    const uint32_t man = x & 0x7fffffu;
    if (e == 0xffu) return static_cast<uint16_t>(sign | 0x7c00u | (man ? 0x200u : 0u));
    const int32_t he = static_cast<int32_t>(e) - 112;
    if (he >= 31) return static_cast<uint16_t>(sign | 0x7c00u);
    uint32_t sig = (e == 0) ? man : (man | 0x800000u);
    int shift;
    uint32_t base;
    if (he >= 1) { shift = 13; base = static_cast<uint32_t>(he) << 10; sig &= 0x7fffffu; }
    else { shift = 14 - he; base = 0; if (shift > 31) return static_cast<uint16_t>(sign); }
    const uint32_t q = sig >> shift, rem = sig & ((1u << shift) - 1u), half = 1u << (shift - 1);
    uint32_t r = base + q;
    if (rem > half || (rem == half && (q & 1u))) ++r;
    if (r >= 0x7c00u) r = 0x7c00u;
    return static_cast<uint16_t>(sign | r);
}
static uint16_t host_f32_to_bf16(float f, int trunc)
{
    uint32_t x;
    memcpy(&x, &f, 4);
    if (trunc) return static_cast<uint16_t>(x >> 16);
    if ((x & 0x7f800000u) == 0x7f800000u && (x & 0x7fffffu)) return static_cast<uint16_t>((x >> 16) | 0x40u);
    x += 0x7fffu + ((x >> 16) & 1u);
    return static_cast<uint16_t>(x >> 16);
}

TL_API tl_status tl_convert_host(const float* src, int64_t n, tl_dtype dtype, tl_rounding rounding, void* dst)
{
    if (n < 0 || (n && (!src || !dst))) return fail(TL_ERR_INVALID_ARG, "bad argument");
    switch (dtype) {
    case TL_DTYPE_FP32: memcpy(dst, src, static_cast<size_t>(n) * 4); break;
    case TL_DTYPE_FP16:
        for (int64_t i = 0; i < n; ++i) static_cast<uint16_t*>(dst)[i] = host_f32_to_f16(src[i]);
        break;
    case TL_DTYPE_BF16:
        for (int64_t i = 0; i < n; ++i)
            static_cast<uint16_t*>(dst)[i] = host_f32_to_bf16(src[i], rounding == TL_ROUND_TRUNCATE);
        break;
    default: return fail(TL_ERR_UNSUPPORTED, "host conversion to this dtype is not provided");
    }
    return TL_SUCCESS;
}

// ---- timers ------------------------------------------------------------------------------------------
TL_API tl_status tl_timer_create(tl_timer** t)
{
    if (!t) return fail(TL_ERR_INVALID_ARG, "NULL out-pointer");
    tl_timer* x = new (std::nothrow) tl_timer();
    if (!x) return fail(TL_ERR_ALLOC, "timer allocation failed");
    if (cudaEventCreate(&x->start) != cudaSuccess || cudaEventCreate(&x->stop) != cudaSuccess) {
        delete x;
        return fail(TL_ERR_CUDA, "cudaEventCreate");
    }
    *t = x;
    return TL_SUCCESS;
}
TL_API tl_status tl_timer_start(tl_timer* t, void* s) { TL_CUDA_TRY(cudaEventRecord(t->start, S(s))); return TL_SUCCESS; }
TL_API tl_status tl_timer_stop(tl_timer* t, void* s) { TL_CUDA_TRY(cudaEventRecord(t->stop, S(s))); return TL_SUCCESS; }
TL_API tl_status tl_timer_elapsed_ms(tl_timer* t, float* ms)
{
    TL_CUDA_TRY(cudaEventSynchronize(t->stop));
    TL_CUDA_TRY(cudaEventElapsedTime(ms, t->start, t->stop));
    return TL_SUCCESS;
}
TL_API tl_status tl_timer_destroy(tl_timer* t)
{
    if (!t) return TL_SUCCESS;
    cudaEventDestroy(t->start);
    cudaEventDestroy(t->stop);
    delete t;
    return TL_SUCCESS;
}

TL_API tl_status tl_set_kernel_timing(tl_handle* h, int enable)
{
    if (h && h->host_only) return host_only_refused();
    if (!h) return fail(TL_ERR_INVALID_ARG, "handle is NULL");
    std::lock_guard<std::mutex> lock(h->mu);
    if (enable && h->tev.empty()) {
        int prev = 0;
        TL_CUDA_TRY(cudaGetDevice(&prev));
        TL_CUDA_TRY(cudaSetDevice(h->device));
        h->tev.resize(2 * kTimingPairs, nullptr);
        cudaError_t ce = cudaSuccess;
        for (auto& e : h->tev)
            if ((ce = cudaEventCreate(&e)) != cudaSuccess) break;
        cudaSetDevice(prev);
        if (ce != cudaSuccess) {
            for (auto& x : h->tev) if (x) cudaEventDestroy(x);
            h->tev.clear();
            return cuda_fail(ce, "cudaEventCreate");
        }
    }
    if (!enable) {
        tl_status st = timing_fold(h);
        if (st != TL_SUCCESS) return st;
    }
    h->timing = enable != 0;
    return TL_SUCCESS;
}

TL_API tl_status tl_kernel_timing(tl_handle* h, double* total_ms, int64_t* launches, int reset)
{
    if (h && h->host_only) return host_only_refused();
    if (!h) return fail(TL_ERR_INVALID_ARG, "handle is NULL");
    std::lock_guard<std::mutex> lock(h->mu);
    tl_status st = timing_fold(h);
    if (st != TL_SUCCESS) return st;
    if (total_ms) *total_ms = h->timing_ms;
    if (launches) *launches = h->timing_count;
    if (reset) {
        h->timing_ms = 0.0;
        h->timing_count = 0;
    }
    return TL_SUCCESS;
}

TL_API tl_status tl_launch_count(tl_handle* h, int64_t* n)
{
    if (!h || !n) return fail(TL_ERR_INVALID_ARG, "NULL argument");
    *n = h->launches;
    return TL_SUCCESS;
}

TL_API tl_status tl_device_status(tl_handle* h, void* stream)
{
    if (h && h->host_only) return host_only_refused();
    if (!h) return fail(TL_ERR_INVALID_ARG, "handle is NULL");
    cudaError_t e = cudaStreamSynchronize(S(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    int v = 0;
    TL_CUDA_TRY(cudaMemcpy(&v, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (v) {
        TL_CUDA_TRY(cudaMemset(h->d_err, 0, sizeof(int)));
        // a launch that gave up may have left split-k arrival counters mid-count: the next launch
        // expects them at zero
        if (h->counters) TL_CUDA_TRY(cudaMemset(h->counters, 0, h->counters_len * sizeof(int)));
        char buf[128];
        snprintf(buf, sizeof(buf), "device wait timed out (role mask 0x%x)", v);
        return fail(TL_ERR_TIMEOUT, buf);
    }
    return TL_SUCCESS;
}

TL_API tl_status tl_set_wait_timeout(tl_handle* h, uint32_t ms)
{
    if (!h || ms == 0) return fail(TL_ERR_INVALID_ARG, "bad argument");
    h->timeout_ns = static_cast<uint64_t>(ms) * 1000000ull;
    return TL_SUCCESS;
}

TL_API tl_status tl_set_trace(tl_handle* h, void* buf, int64_t bytes)
{
    if (!h || bytes < 0 || (buf != nullptr && (reinterpret_cast<uintptr_t>(buf) % 8) != 0))
        return fail(TL_ERR_INVALID_ARG, "bad argument");
    std::lock_guard<std::mutex> lk(h->mu);
    h->trace = (buf != nullptr && bytes > 0) ? static_cast<unsigned long long*>(buf) : nullptr;
    h->trace_bytes = h->trace ? bytes : 0;
    return TL_SUCCESS;
}

}  // extern "C"
