// gemm_tc.cu -- the tensor-core GEMM for sm_103a.
//
// D(m,n) = alpha * sum_k op(A)(m,k) op(B)(k,n) + beta * C(m,n), column-major, fp32 accumulation in
// TMEM.  This is the GB300 counterpart of TensileLite's generated MFMA kernel
// (src/gemmMfmaKernelWriter.h:24-2073): the reference's fetch waves (global -> LDS ring,
// :408-432/:1226-1400) become one TMA producer warp feeding a shared-memory ring guarded by
// full/empty mbarriers; its math waves (LDS -> VGPR -> MFMA into AccVGPRs, :433-466/:1403-1547)
// become one thread issuing tcgen05.mma from shared-memory descriptors into a TMEM accumulator;
// its fused epilogue (beta*C pre-scaled, fma(alpha, acc, beta*C), convert, store; :1572-1768,
// :1822-1906) becomes four warps draining TMEM with tcgen05.ld while the next tile accumulates into
// the second TMEM buffer.
//
// Roles (192 threads, one CTA per SM, persistent over work units):
//   warp 0     TMA producer: per k-block one box of B (128 n-rows) and one of A (bm m-rows)
//   warp 1     TMEM allocator + MMA issuer (lane 0): 4 tcgen05.mma per k-block, commit -> empty
//   warps 2-5  epilogue: TMEM lane = problem n, TMEM column = problem m, so each thread owns a
//              contiguous run of m for one n -- column-major D rows are written as 16-byte vectors.
// The problem's B^T is the MMA "A" operand (M = 128 along n) and A is the MMA "B" operand
// (N = bm along m).  K-major operands (TN, the reference's layout) and MN-major operands (NN/NT)
// are both read straight from global memory by TMA with 128-byte swizzling; no transpose pass.
//
// Work unit = (tile, k-split).  Split-k partials go to a workspace; the last CTA to finish a tile
// (arrival counter) sums the partials in split order and runs the epilogue, so results do not
// depend on scheduling.  The grouped variant walks a problem table with per-problem TMA maps.
//
// Every mbarrier wait is bounded (globaltimer); on expiry the kernel sets *err and returns.



#include "gemm_tc_kernel.cuh"

#include <mutex>

namespace tl {
namespace tc {

// instantiated in the generated instance units (one per operand kind, cluster size, epilogue)
#define TL_TC_EXTERN(K, TD, CL, E) extern template tl_status launch_kernel<K, TD, CL, E>(const TcKernelParams&, int, size_t, cudaStream_t);
#define TL_TC_EXTERN_CL(K, CL)                                                                                 \
    TL_TC_EXTERN(K, float, CL, false) TL_TC_EXTERN(K, __half, CL, false) TL_TC_EXTERN(K, __nv_bfloat16, CL, false) \
    TL_TC_EXTERN(K, float, CL, true) TL_TC_EXTERN(K, __half, CL, true) TL_TC_EXTERN(K, __nv_bfloat16, CL, true)    \
    TL_TC_EXTERN(K, __nv_fp8_e4m3, CL, true)                                                                  \
    extern template int max_clusters<K, float, CL>(size_t);                                                   \
    extern template int max_clusters<K, __half, CL>(size_t);                                                  \
    extern template int max_clusters<K, __nv_bfloat16, CL>(size_t);
TL_TC_EXTERN_CL(0, 1)
TL_TC_EXTERN_CL(0, 2)
TL_TC_EXTERN_CL(0, 4)
TL_TC_EXTERN_CL(1, 1)
TL_TC_EXTERN_CL(1, 2)
TL_TC_EXTERN_CL(1, 4)
#undef TL_TC_EXTERN_CL
#undef TL_TC_EXTERN

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(ptr);
    });
    return fn;
}

// Parallel split-k reduction: on unless TL_PAR_REDUCE=0 in the environment.
bool par_reduce_enabled()
{
    static const bool on = [] {
        const char* e = getenv("TL_PAR_REDUCE");
        return !(e && e[0] == '0');
    }();
    return on;
}

// TMA-store epilogue: on unless TL_TMA_STORE=0 in the environment.
bool tma_store_enabled()
{
    static const bool on = [] {
        const char* e = getenv("TL_TMA_STORE");
        return !(e && e[0] == '0');
    }();
    return on;
}

// A CTA's last tile is written with direct stores unless TL_LAST_DIRECT=0 in the environment.
bool last_direct_enabled()
{
    static const bool on = [] {
        const char* e = getenv("TL_LAST_DIRECT");
        return !(e && e[0] == '0');
    }();
    return on;
}

// Programmatic dependent launch for the tensor-core kernel: on unless TL_PDL=0 in the environment.
bool pdl_enabled()
{
    static const bool on = [] {
        const char* e = getenv("TL_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

template <int CL>
tl_status dispatch_cl(int in_dtype, int out_dtype, const TcKernelParams& kp, int grid, size_t smem, cudaStream_t s)
{
    const int kind = (in_dtype == TL_DTYPE_FP8_E4M3) ? 1 : 0;
    if (kp.epi_on) {
        // the fused-epilogue kernels (they also write every fp8 output)
        if (kind == 0) {
            if (out_dtype == TL_DTYPE_FP32) return launch_kernel<0, float, CL, true>(kp, grid, smem, s);
            if (out_dtype == TL_DTYPE_FP16) return launch_kernel<0, __half, CL, true>(kp, grid, smem, s);
            if (out_dtype == TL_DTYPE_BF16) return launch_kernel<0, __nv_bfloat16, CL, true>(kp, grid, smem, s);
            if (out_dtype == TL_DTYPE_FP8_E4M3) return launch_kernel<0, __nv_fp8_e4m3, CL, true>(kp, grid, smem, s);
        } else {
            if (out_dtype == TL_DTYPE_FP32) return launch_kernel<1, float, CL, true>(kp, grid, smem, s);
            if (out_dtype == TL_DTYPE_FP16) return launch_kernel<1, __half, CL, true>(kp, grid, smem, s);
            if (out_dtype == TL_DTYPE_BF16) return launch_kernel<1, __nv_bfloat16, CL, true>(kp, grid, smem, s);
            if (out_dtype == TL_DTYPE_FP8_E4M3) return launch_kernel<1, __nv_fp8_e4m3, CL, true>(kp, grid, smem, s);
        }
        return fail(TL_ERR_UNSUPPORTED, "tcgen05 kernel: unsupported output type");
    }
    if (kind == 0) {
        if (out_dtype == TL_DTYPE_FP32) return launch_kernel<0, float, CL>(kp, grid, smem, s);
        if (out_dtype == TL_DTYPE_FP16) return launch_kernel<0, __half, CL>(kp, grid, smem, s);
        if (out_dtype == TL_DTYPE_BF16) return launch_kernel<0, __nv_bfloat16, CL>(kp, grid, smem, s);
    } else {
        if (out_dtype == TL_DTYPE_FP32) return launch_kernel<1, float, CL>(kp, grid, smem, s);
        if (out_dtype == TL_DTYPE_FP16) return launch_kernel<1, __half, CL>(kp, grid, smem, s);
        if (out_dtype == TL_DTYPE_BF16) return launch_kernel<1, __nv_bfloat16, CL>(kp, grid, smem, s);
    }
    return fail(TL_ERR_UNSUPPORTED, "tcgen05 kernel: unsupported output type");
}

template <int CL>
int max_clusters_for(int in_dtype, int out_dtype, size_t smem)
{
    if (in_dtype != TL_DTYPE_FP8_E4M3)
        return out_dtype == TL_DTYPE_FP32   ? max_clusters<0, float, CL>(smem)
               : out_dtype == TL_DTYPE_FP16 ? max_clusters<0, __half, CL>(smem)
                                            : max_clusters<0, __nv_bfloat16, CL>(smem);
    return out_dtype == TL_DTYPE_FP32   ? max_clusters<1, float, CL>(smem)
           : out_dtype == TL_DTYPE_FP16 ? max_clusters<1, __half, CL>(smem)
                                        : max_clusters<1, __nv_bfloat16, CL>(smem);
}

// Persistent workers of a launch: CTAs (cl 1) or co-resident clusters of cl CTAs (2: a CTA pair,
// 4: two pairs sharing the m-side operand).
int persistent_workers(int in_dtype, int out_dtype, int cl, int ctas, int sm_count, size_t smem)
{
    if (cl == 1) return ctas > 0 ? ctas : sm_count;
    if (ctas > 0) return ctas / cl > 0 ? ctas / cl : 1;
    const int maxc = cl == 2 ? max_clusters_for<2>(in_dtype, out_dtype, smem) : max_clusters_for<4>(in_dtype, out_dtype, smem);
    return maxc > 0 ? maxc : sm_count / cl;
}

// Grid: one CTA per SM (cl 1) or as many co-resident clusters as fit, never more than the work.
tl_status dispatch(int in_dtype, int out_dtype, int cl, const TcKernelParams& kp_in, int ctas, int sm_count,
                   int64_t total_work, size_t smem, cudaStream_t s, int64_t trace_bytes)
{
    int workers = persistent_workers(in_dtype, out_dtype, cl, ctas, sm_count, smem);
    if (workers > total_work) workers = static_cast<int>(total_work);
    if (workers < 1) workers = 1;
    const int grid = (cl == 1 ? 1 : (cl == 2 ? 2 : 4)) * workers;
    const TcKernelParams* kp = &kp_in;
    TcKernelParams untraced;
    if (kp_in.trace != nullptr &&
        static_cast<int64_t>(grid) * TL_TRACE_SLOTS * static_cast<int64_t>(sizeof(unsigned long long)) > trace_bytes) {
        untraced = kp_in;             // the timeline buffer cannot hold this grid: record nothing
        untraced.trace = nullptr;
        kp = &untraced;
    }
    if (cl == 1) return dispatch_cl<1>(in_dtype, out_dtype, *kp, grid, smem, s);
    if (cl == 2) return dispatch_cl<2>(in_dtype, out_dtype, *kp, grid, smem, s);
    return dispatch_cl<4>(in_dtype, out_dtype, *kp, grid, smem, s);
}

uint32_t make_idesc(int in_dtype, int n_mn_major, int m_mn_major, int bm, int cg)
{
    uint32_t d = 1u << 4;                                  // accumulator F32
    uint32_t t = (in_dtype == TL_DTYPE_BF16) ? 1u : 0u;    // kind::f16: 0 F16, 1 BF16; f8f6f4: 0 E4M3
    d |= t << 7;                                           // A (problem B^T) type
    d |= t << 10;                                          // B (problem A) type
    d |= static_cast<uint32_t>(n_mn_major & 1) << 15;      // A major: 0 K, 1 MN
    d |= static_cast<uint32_t>(m_mn_major & 1) << 16;      // B major
    d |= static_cast<uint32_t>(bm >> 3) << 17;             // N >> 3
    d |= static_cast<uint32_t>((kTcTileN * cg) >> 4) << 24;  // M >> 4 (256 for a CTA pair)
    return d;
}

void desc_params(int in_dtype, int mn_major, uint32_t& lbo, uint32_t& kstep)
{
    const int es = dtype_bytes(in_dtype);
    const int W = kTcRowBytes / es;          // elements per 128-byte row == depth_u
    const int umma_k = 32 / es;              // 16 for 16-bit, 32 for fp8
    if (!mn_major) {
        lbo = 16;                            // unused for swizzled K-major
        kstep = umma_k * es;                 // 32 bytes along the swizzled row
    } else {
        lbo = static_cast<uint32_t>(W) * kTcRowBytes;   // next MN chunk of W elements
        kstep = umma_k * kTcRowBytes;                    // umma_k rows of 128 bytes
    }
}

}  // namespace tc

using namespace tc;

size_t tc_smem_bytes(int bm, int stages)
{
    // ring + output staging + 1024 bytes to align the ring + barriers/flags (with margin)
    return static_cast<size_t>(stages) * (kTcTileN * kTcRowBytes + bm * kTcRowBytes) + kTcEpiStageBytes + 1024 + 512;
}

int tc_workers(int in_dtype, int out_dtype, int cl, int bm, int stages, int sm_count)
{
    const int cta_group = cl >= 2 ? 2 : 1;
    return persistent_workers(in_dtype, out_dtype, cl, 0, sm_count, tc_smem_bytes(bm / cta_group, stages));
}

int tc_tmem_cols(int bm) { return (2 * bm <= 128) ? 128 : (2 * bm <= 256 ? 256 : 512); }

tl_status tc_encode_operand(CUtensorMap* tm, int in_dtype, const TcOperand& op, int64_t K, int64_t batch,
                            int box_rows)
{
    EncodeTiledFn enc = get_encode_fn();
    if (!enc) return fail(TL_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
    const int es = dtype_bytes(in_dtype);
    const int W = kTcRowBytes / es;
    CUtensorMapDataType dt = in_dtype == TL_DTYPE_BF16   ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                             : in_dtype == TL_DTYPE_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                         : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    cuuint64_t dims[3];
    cuuint64_t strides[2];
    cuuint32_t box[3];
    cuuint32_t estr[3] = {1, 1, 1};
    if (!op.mn_major) {
        dims[0] = static_cast<cuuint64_t>(K);
        dims[1] = static_cast<cuuint64_t>(op.rows);
        box[0] = W;
        box[1] = box_rows;
    } else {
        dims[0] = static_cast<cuuint64_t>(op.rows);
        dims[1] = static_cast<cuuint64_t>(K);
        box[0] = W;
        box[1] = W;
    }
    dims[2] = static_cast<cuuint64_t>(batch);
    box[2] = 1;
    strides[0] = static_cast<cuuint64_t>(op.ld) * es;
    cuuint64_t bstride = static_cast<cuuint64_t>(op.batch_stride) * es;
    if (batch <= 1) bstride = ((strides[0] * dims[1]) + 15) & ~cuuint64_t(15);
    strides[1] = bstride;
    CUresult r = enc(tm, dt, 3, const_cast<void*>(op.ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char buf[256];
        snprintf(buf, sizeof(buf),
                 "cuTensorMapEncodeTiled failed (%d): dims {%llu,%llu,%llu} strides {%llu,%llu} box {%u,%u}",
                 static_cast<int>(r), (unsigned long long)dims[0], (unsigned long long)dims[1],
                 (unsigned long long)dims[2], (unsigned long long)strides[0], (unsigned long long)strides[1], box[0],
                 box[1]);
        return fail(TL_ERR_INVALID_ARG, buf);
    }
    return TL_SUCCESS;
}

// Tensor map of the output for TMA stores: boxes of 128 bytes along m by 32 rows (n), 128-byte
// swizzle.  False when TMA cannot address D (alignment of the base, ldd or batch stride).
bool tc_encode_output(CUtensorMap* tm, int out_dtype, void* D, int64_t M, int64_t N, int64_t ldd, int64_t batch,
                      int64_t stride_d)
{
    EncodeTiledFn enc = get_encode_fn();
    if (!enc || !D) return false;
    const int es = dtype_bytes(out_dtype);
    if ((reinterpret_cast<uintptr_t>(D) & 15) || (ldd * es) % 16 || (batch > 1 && (stride_d * es) % 16)) return false;
    const CUtensorMapDataType dt = out_dtype == TL_DTYPE_FP32   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : out_dtype == TL_DTYPE_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                   : out_dtype == TL_DTYPE_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                                : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    cuuint64_t dims[3] = {static_cast<cuuint64_t>(M), static_cast<cuuint64_t>(N), static_cast<cuuint64_t>(batch)};
    cuuint64_t strides[2] = {static_cast<cuuint64_t>(ldd) * es,
                             batch > 1 ? static_cast<cuuint64_t>(stride_d) * es
                                       : ((static_cast<cuuint64_t>(ldd) * es * N) + 15) & ~cuuint64_t(15)};
    cuuint32_t box[3] = {static_cast<cuuint32_t>(kTcRowBytes / es), 32, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    return enc(tm, dt, 3, D, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
               CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The caller's D for a transposed output: the kernel's n runs along D's rows (dimension 0, N of
// the launch) and its m along D's columns; boxes of 32 x 32 elements, one epilogue warp's rows by
// one 32-column chunk, unswizzled (a 64- or 128-byte inner extent).
bool tc_encode_output_t(CUtensorMap* tm, int out_dtype, void* D, int64_t rows, int64_t cols, int64_t ldd,
                        int64_t batch, int64_t stride_d)
{
    EncodeTiledFn enc = get_encode_fn();
    if (!enc || !D) return false;
    if (out_dtype != TL_DTYPE_FP32 && out_dtype != TL_DTYPE_FP16 && out_dtype != TL_DTYPE_BF16) return false;
    const int es = dtype_bytes(out_dtype);
    if ((reinterpret_cast<uintptr_t>(D) & 15) || (ldd * es) % 16 || (batch > 1 && (stride_d * es) % 16)) return false;
    const CUtensorMapDataType dt = out_dtype == TL_DTYPE_FP32   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                   : out_dtype == TL_DTYPE_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                                : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    cuuint64_t dims[3] = {static_cast<cuuint64_t>(rows), static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(batch)};
    cuuint64_t strides[2] = {static_cast<cuuint64_t>(ldd) * es,
                             batch > 1 ? static_cast<cuuint64_t>(stride_d) * es
                                       : ((static_cast<cuuint64_t>(ldd) * es * cols) + 15) & ~cuuint64_t(15)};
    cuuint32_t box[3] = {32, 32, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    return enc(tm, dt, 3, D, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

tl_status tc_gemm_launch(const TcLaunch& L, cudaStream_t stream, int64_t* launches)
{
    TcKernelParams kp;
    memset(&kp, 0, sizeof(kp));
    tl_status st;
    const int pieces = L.pieces < 1 ? 1 : L.pieces;
    const int cg = (L.cg == 2 || L.cg == 4) ? L.cg : 1;     // CTAs per cluster
    const int cta_group = cg >= 2 ? 2 : 1;
    for (int i = 0; i < pieces; ++i) {
        if ((st = tc_encode_operand(&kp.tmN[i], L.in_dtype, L.opN[i], L.K, L.batch, kTcTileN)) != TL_SUCCESS) return st;
        if ((st = tc_encode_operand(&kp.tmM[i], L.in_dtype, L.opM[i], L.K, L.batch, L.bm / cg)) != TL_SUCCESS) return st;
    }
    // products per k-block, smallest first: 2-piece split -> A1B0, A0B1, A0B0;
    // 3-piece split -> A2B0, A1B1, A0B2, A1B0, A0B1, A0B0
    static const uint8_t t3m[3] = {1, 0, 0}, t3n[3] = {0, 1, 0};
    static const uint8_t t6m[6] = {2, 1, 0, 1, 0, 0}, t6n[6] = {0, 1, 2, 0, 1, 0};
    if (pieces == 1) { kp.nterms = 1; kp.term_m[0] = kp.term_n[0] = 0; }
    else if (pieces == 2) { kp.nterms = 3; for (int i = 0; i < 3; ++i) { kp.term_m[i] = t3m[i]; kp.term_n[i] = t3n[i]; } }
    else { kp.nterms = 6; for (int i = 0; i < 6; ++i) { kp.term_m[i] = t6m[i]; kp.term_n[i] = t6n[i]; } }
    const int W = kTcRowBytes / dtype_bytes(L.in_dtype);
    kp.group = nullptr;
    kp.D = L.D;
    kp.C = L.C;
    kp.ldd = L.ldd;
    kp.ldc = L.ldc;
    kp.stride_d = L.stride_d;
    kp.stride_c = L.stride_c;
    kp.M = static_cast<int>(L.M);
    kp.N = static_cast<int>(L.N);
    kp.K = static_cast<int>(L.K);
    kp.batch = static_cast<int>(L.batch);
    kp.alpha = L.alpha;
    kp.beta = L.beta;
    kp.bm = L.bm;
    kp.stages = L.stages;
    kp.split_k = L.split_k;
    kp.raster = L.raster;
    kp.tiles_m = static_cast<int>((L.M + L.bm - 1) / L.bm);
    kp.tile_rows = kTcTileN * cg;
    kp.tiles_n = static_cast<int>((L.N + kp.tile_rows - 1) / kp.tile_rows);
    kp.num_kb = static_cast<int>((L.K + W - 1) / W);
    kp.kb_elems = W;
    kp.promote_kb = L.promote_k > 0 ? static_cast<int>((L.promote_k + W - 1) / W) : 0;
    const size_t smem = tc_smem_bytes(L.bm / cta_group, L.stages);
    const int64_t tiles = static_cast<int64_t>(kp.tiles_m) * kp.tiles_n * L.batch;
    kp.bal_kb = 0;
    kp.bal_workers = 0;
    kp.bal_stride = 0;
    if (L.split_k > 1) {
        kp.split_units = tiles * L.split_k;
        kp.split_tiles = tiles;
        kp.tail_split = L.split_k;
        kp.total_work = tiles * L.split_k;
    } else {
        kp.split_units = 0;
        kp.split_tiles = 0;
        kp.tail_split = 1;
        kp.total_work = tiles;
        const int workers = persistent_workers(L.in_dtype, L.out_dtype, cg, L.ctas, L.sm_count, smem);
        const int64_t rem = tiles % workers, full = tiles / workers;
        const size_t slab = static_cast<size_t>(kTcTileN) * L.bm * sizeof(float);
        // measured on GB300: a piece needs about 48 k-blocks (balanced) or 16 (uniform slices) to
        // amortise its partial-tile round trip; shorter pieces lose more than the idle workers
        const int64_t R = rem * kp.num_kb;
        const int64_t Wmax = std::min<int64_t>(std::min<int64_t>(workers, 8 * rem), R / 2);
        // tail_split -1 asks for the balanced split whatever the piece length
        // (the piece length R / Wmax is only formed once Wmax > 1: no whole last wave, or a single
        // tile of one k-block, leaves Wmax at 0)
        const bool balanced = rem > 0 && Wmax > 1 && Wmax >= rem && L.promote_k == 0 &&
                              (L.tail_split == -1 || (L.tail_split == 0 && R / Wmax >= 48));
        if (balanced && L.workspace) {
            // balanced split (automatic, long k): the k-blocks of the last partial wave's tiles
            // are cut into equal contiguous ranges, one per worker (at most 8 pieces per tile); a
            // range covers at most two tiles.  The pieces run first so their reductions overlap
            // the whole tiles that follow; with no whole wave after them the reduction is exposed,
            // so then the split must save a good part of a tile.
            int64_t Wb = Wmax;
            while (Wb >= rem) {
                const int64_t per = R / Wb;
                const int64_t maxS = (kp.num_kb + per - 1) / per + 1;
                const size_t need = static_cast<size_t>(rem) * cg * maxS * slab;
                if (need <= L.workspace_bytes && static_cast<size_t>(rem) * cg <= L.counters_len) break;
                --Wb;
            }
            const int64_t saved = Wb >= rem ? kp.num_kb - (R + Wb - 1) / Wb : 0;
            if (Wb >= rem && Wb > 1 &&
                (L.tail_split == -1 || saved >= (full >= 1 ? 2 : std::max<int64_t>(8, kp.num_kb / 3)))) {
                const int64_t per = R / Wb;
                kp.bal_kb = R;
                kp.bal_workers = static_cast<int>(Wb);
                kp.bal_stride = workers;
                kp.split_tiles = rem;
                kp.split_units = 2 * static_cast<int64_t>(workers);
                kp.tail_split = static_cast<int>((kp.num_kb + per - 1) / per + 1);   // slab stride
                kp.total_work = 2 * static_cast<int64_t>(workers) + (tiles - rem);
            }
        } else if (L.tail_split != 1 && L.tail_split != -1 && L.workspace && tiles > workers && rem > 0 &&
                   2 * rem <= workers) {
            // uniform tail split (explicit S, or automatic): the last partial wave's tiles are cut
            // into S equal k-slices, scheduled first
            int S = L.tail_split > 1 ? L.tail_split : static_cast<int>(std::min<int64_t>(workers / rem, kp.num_kb / 16));
            if (S > kp.num_kb) S = kp.num_kb;
            if (S > 8) S = 8;
            const size_t need = static_cast<size_t>(rem) * cg * S * slab;
            if (S >= 2 && static_cast<size_t>(rem) * cg <= L.counters_len && need <= L.workspace_bytes) {
                kp.split_tiles = rem;
                kp.split_units = rem * S;
                kp.tail_split = S;
                kp.total_work = rem * S + (tiles - rem);
            }
        }
    }
    kp.n_mn_major = L.opN[0].mn_major;
    kp.m_mn_major = L.opM[0].mn_major;
    kp.idesc = make_idesc(L.in_dtype, kp.n_mn_major, kp.m_mn_major, L.bm, cta_group);
    desc_params(L.in_dtype, kp.n_mn_major, kp.n_lbo, kp.n_kstep);
    desc_params(L.in_dtype, kp.m_mn_major, kp.m_lbo, kp.m_kstep);
    kp.out_trunc = L.out_trunc;
    kp.epi_on = L.epi_on;
    kp.epi_dscale = L.epi_dscale;
    kp.epi_bias = L.epi_bias;
    kp.epi_amax = L.epi_amax;
    kp.epi_bias_dtype = L.epi_bias_dtype;
    kp.epi_act = L.epi_act;
    // all split units in the first round of the persistent schedule: parallel reduction
    {
        const int workers = persistent_workers(L.in_dtype, L.out_dtype, cg, L.ctas, L.sm_count, smem);
        kp.par_reduce = (kp.split_units > 0 && kp.bal_kb == 0 && kp.split_units <= workers && par_reduce_enabled()) ? 1 : 0;
    }
    // whole tiles leave through TMA stores (not with promotion, which drains chains into registers)
    // (an fp8 output's 128-byte box is 128 columns wide: only tiles made of whole boxes)
    kp.out_t = L.out_t;
    if (L.out_t)
        kp.tma_store = (L.promote_k == 0 && tma_store_enabled() &&
                        tc_encode_output_t(&kp.tmD, L.out_dtype, L.D, L.N, L.M, L.ldd, L.batch, L.stride_d))
                           ? 1
                           : 0;
    else
        kp.tma_store = (L.promote_k == 0 && tma_store_enabled() && (L.out_dtype != TL_DTYPE_FP8_E4M3 || L.bm % 128 == 0) &&
                        tc_encode_output(&kp.tmD, L.out_dtype, L.D, L.M, L.N, L.ldd, L.batch, L.stride_d))
                           ? 1
                           : 0;
    kp.direct_last = last_direct_enabled() ? 1 : 0;
    kp.narrow = (kp.total_work < (int64_t(1) << 31) && tiles < (int64_t(1) << 31) &&
                 static_cast<int64_t>(kp.num_kb) * (kp.tail_split + 1) < (int64_t(1) << 31))
                    ? 1
                    : 0;
    kp.ws = L.workspace;
    kp.counters = L.counters;
    kp.err = L.err;
    kp.timeout_ns = L.timeout_ns;
    kp.debug_skip_loads = (L.debug_flags & TL_DEBUG_SKIP_LOADS) ? 1 : 0;
    kp.trace = L.trace;
    st = dispatch(L.in_dtype, L.out_dtype, cg, kp, L.ctas, L.sm_count, kp.total_work, smem, stream, L.trace_bytes);
    if (st == TL_SUCCESS && launches) ++*launches;
    return st;
}

tl_status tc_grouped_launch(const TcGroupLaunch& G, cudaStream_t stream, int64_t* launches)
{
    TcKernelParams kp;
    memset(&kp, 0, sizeof(kp));
    kp.group = G.d_entries;
    kp.group_units = G.d_units;
    kp.direct_last = last_direct_enabled() ? 1 : 0;
    kp.bm = G.bm;
    kp.stages = G.stages;
    kp.split_k = 1;
    kp.nterms = 1;
    kp.total_work = G.total_tiles;
    kp.split_units = 0;
    kp.split_tiles = 0;
    kp.tail_split = 1;
    kp.kb_elems = kTcRowBytes / dtype_bytes(G.in_dtype);
    kp.stride_c = 0;
    kp.stride_d = 0;
    kp.n_mn_major = G.n_mn_major;
    kp.m_mn_major = G.m_mn_major;
    const int cg = (G.cg == 2 || G.cg == 4) ? G.cg : 1;     // CTAs per cluster
    const int cta_group = cg >= 2 ? 2 : 1;
    kp.tile_rows = kTcTileN * cg;
    kp.idesc = make_idesc(G.in_dtype, G.n_mn_major, G.m_mn_major, G.bm, cta_group);
    desc_params(G.in_dtype, G.n_mn_major, kp.n_lbo, kp.n_kstep);
    desc_params(G.in_dtype, G.m_mn_major, kp.m_lbo, kp.m_kstep);
    kp.out_trunc = G.out_trunc;
    kp.err = G.err;
    kp.timeout_ns = G.timeout_ns;
    const size_t smem = tc_smem_bytes(G.bm / cta_group, G.stages);
    tl_status st = dispatch(G.in_dtype, G.out_dtype, cg, kp, G.ctas, G.sm_count, G.total_tiles, smem, stream, 0);
    if (st == TL_SUCCESS && launches) ++*launches;
    return st;
}

}  // namespace tl
