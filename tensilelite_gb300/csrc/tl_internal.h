// tl_internal.h -- types shared by the C-ABI layer (tl_api.cpp) and the kernel launchers (*.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tensilelite.h"

namespace tl {

// ---- error reporting ------------------------------------------------------------------------------
void set_error(const std::string& msg);
tl_status fail(tl_status st, const std::string& msg);
tl_status cuda_fail(cudaError_t e, const char* what);
#define TL_CUDA_TRY(call)                                  \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return ::tl::cuda_fail(e_, #call); \
    } while (0)

inline int dtype_bytes(int dt)
{
    switch (dt) {
    case TL_DTYPE_FP32: return 4;
    case TL_DTYPE_FP16: return 2;
    case TL_DTYPE_BF16: return 2;
    case TL_DTYPE_FP8_E4M3: return 1;
    default: return 0;
    }
}

// ---- tcgen05 GEMM launch description ----------------------------------------------------------------
constexpr int kTcMaxStages = 8;
constexpr int kTcTileN = 128;          // tcgen05 M extent: problem n rows on TMEM lanes
constexpr int kTcRowBytes = 128;       // one swizzle row: depth_u * element size
constexpr int kTcEpiStageBytes = 4 * 32 * 128;   // output staging of the 4 epilogue warps (TMA stores)
constexpr int kTcThreads = 192;        // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue

// One operand's TMA view: K-major (rows x k, k contiguous) or MN-major (k rows of contiguous rows).
struct TcOperand {
    const void* ptr;
    int64_t rows;      // n (opN = problem B) or m (opM = problem A)
    int64_t ld;        // elements
    int64_t batch_stride;
    int mn_major;      // 1: rows contiguous in memory
};

// Per-problem table entry for the grouped kernel (device memory; CUtensorMap members fix the alignment).
struct TcGroupEntry {   // aligned like CUtensorMap
    CUtensorMap tmN;   // problem B view
    CUtensorMap tmM;   // problem A view
    void* D;
    const void* C;
    int64_t ldd, ldc;
    int32_t M, N, K;
    int32_t tiles_m, tiles_n;
    float alpha, beta;
    int32_t tma_store;   // tmD describes D: whole tiles leave through TMA stores
    CUtensorMap tmD;     // problem D, boxes of 128 bytes x 32 rows
};

struct TcLaunch {
    // operands
    int in_dtype;            // FP16 / BF16 / FP8_E4M3 (BF16 for the fp32 split paths)
    int out_dtype;
    int out_trunc;
    TcOperand opN[3], opM[3];  // operand pieces: [0] the operand (or its bf16 head), [1..2] residuals
    int pieces;              // 1 plain, 2 = bf16x3 (3 products), 3 = bf16x6 (6 products)
    int64_t M, N, K, batch;
    void* D;
    const void* C;
    int64_t ldd, ldc, stride_d, stride_c;
    float alpha, beta;
    // solution
    int bm;                  // tile along m (tcgen05 N): 64..256
    int stages;
    int split_k;
    int raster;
    int ctas;
    int promote_k;           // k elements per TMEM accumulation chain of the A0*B0 product (0: whole k)
    int cg;                  // 1: one CTA per 128-row tile; 2: a CTA pair per 256-row tile
    // runtime
    int* err;
    uint64_t timeout_ns;
    float* workspace;        // split-k partials
    size_t workspace_bytes;
    int* counters;           // split-k arrival counters (zeroed, self-resetting)
    size_t counters_len;
    int tail_split;          // 0 auto, 1 off, S: k splits of the last partial wave's tiles
    int sm_count;
    // fused epilogue: D = act(alpha*acc + beta*C + bias[m]); max |D| into *epi_amax
    const void* epi_bias;
    float* epi_amax;
    float epi_dscale;        // fp8 outputs: multiplied in before the E4M3 rounding
    int epi_bias_dtype;
    int epi_act;
    int epi_on;
    int debug_flags;         // tl_gemm_solution.debug_flags (TL_DEBUG_SKIP_LOADS)
    unsigned long long* trace;   // device timeline (tl_set_trace) or null
    int64_t trace_bytes;
    int out_t;               // D and C hold the transpose of this launch's output (NN run as TT)
};

// Dynamic shared memory of one CTA staging bm_cta m-rows per stage (bm / 2 for a CTA pair).
size_t tc_smem_bytes(int bm_cta, int stages);
// Tensor map of an output for TMA stores (false when TMA cannot address it).
bool tc_encode_output(CUtensorMap* tm, int out_dtype, void* D, int64_t M, int64_t N, int64_t ldd, int64_t batch,
                      int64_t stride_d);
// Persistent workers (CTAs, or co-resident clusters of `cl` CTAs) a tensor-core launch gets.
int tc_workers(int in_dtype, int out_dtype, int cl, int bm, int stages, int sm_count);
int tc_tmem_cols(int bm);
tl_status tc_gemm_launch(const TcLaunch& L, cudaStream_t stream, int64_t* launches);
// Checks a tcgen05 GEMM and fills its launch description without allocating anything; the caller
// provides err, workspace and counters (sizes reported in ws_bytes / counter_count).
tl_status plan_tc_noalloc(int device, int sm_count, size_t smem_optin, const tl_gemm_problem* prob,
                          const tl_gemm_solution* sol, void* D, const void* C, const void* A, const void* B,
                          TcLaunch* L, size_t* ws_bytes, size_t* counter_count);

// Grouped: build per-problem entries (host) and launch over a device table.
struct TcGroupLaunch {
    int in_dtype, out_dtype, out_trunc;
    int n_mn_major, m_mn_major;
    const TcGroupEntry* d_entries;   // device
    const int4* d_units;             // device, one entry per work unit: {problem, tile row, tile column, k-blocks}
    int count;
    int64_t total_tiles;
    int bm, stages, ctas;
    int cg;                          // 1 or 2 (CTA pair)
    int* err;
    uint64_t timeout_ns;
    int sm_count;
};
tl_status tc_encode_operand(CUtensorMap* tm, int in_dtype, const TcOperand& op, int64_t K, int64_t batch,
                            int box_rows);
tl_status tc_grouped_launch(const TcGroupLaunch& G, cudaStream_t stream, int64_t* launches);

// ---- SIMT GEMM -----------------------------------------------------------------------------------
struct SimtLaunch {
    int a_dtype, out_dtype, out_trunc;
    int trans_a, trans_b;
    int64_t M, N, K, batch;
    const void* A; const void* B; const void* C; void* D;
    int64_t lda, ldb, ldc, ldd, sa, sb, sc, sd;
    float alpha, beta;   // alpha already multiplied by fp8 scales
};
tl_status simt_gemm_launch(const SimtLaunch& L, cudaStream_t stream, int64_t* launches);

// ---- auxiliary kernels ------------------------------------------------------------------------------
// x = p0 + p1 (+ p2): each piece the bf16 rounding (RNE) of what the previous pieces leave; p2 may be null.
tl_status aux_split_bf16(const float* src, int64_t rows, int64_t cols, int64_t ld, int64_t batch,
                         int64_t batch_stride, uint16_t* p0, uint16_t* p1, uint16_t* p2, cudaStream_t s,
                         int64_t* launches);
tl_status aux_amax(int src_dtype, const void* src, int64_t n, float* amax_dev, cudaStream_t s, int64_t* launches);
tl_status aux_quant_e4m3(int src_dtype, const void* src, int64_t n, const float* amax_dev, uint8_t* dst,
                         float* scale_out_dev, cudaStream_t s, int64_t* launches);
tl_status aux_error_norms(int dtype_d, const void* D, int64_t ldd, const double* R, const double* W, int64_t ldr,
                          int64_t m, int64_t n, double* out_dev, cudaStream_t s, int64_t* launches);
tl_status aux_fill_pattern(int dtype, void* dst, int64_t count, float code, cudaStream_t s, int64_t* launches);
tl_status aux_scale_c(int out_dtype, int out_trunc, void* D, int64_t ldd, int64_t sd, const void* C, int64_t ldc,
                      int64_t sc, int64_t M, int64_t N, int64_t batch, float beta, cudaStream_t s,
                      int64_t* launches);

}  // namespace tl
