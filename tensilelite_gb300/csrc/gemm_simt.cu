// gemm_simt.cu -- CUDA-core GEMM (FP32 FMA pipes), any input type, fp32 accumulation.
//
// The plain-FP32 counterpart of TensileLite's sgemm path (the fp32 MFMA kernel,
// src/gemmMfmaKernelWriter.h:38-40) and the generic fallback for operands the TMA path cannot
// describe (leading dimensions that are not 16-byte multiples).  128x128 output tile per 256-thread
// CTA, 8x8 outputs per thread in two 4-wide strips per dimension (or, when 128x128 tiles would leave
// most SMs idle, 64x64 tiles with 4x4 outputs per thread), k staged 8 at a time through a
// double-buffered shared-memory ring with the next slab prefetched into registers.  op(A)/op(B) of
// either storage order are read with the thread mapping that keeps the contiguous dimension
// coalesced; edge tiles are zero-filled on load and masked on store.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "tl_internal.h"

namespace tl {
namespace {

constexpr int BK = 8, THREADS = 256;

template <typename T> __device__ __forceinline__ float to_f(T v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<__half>(__half v) { return __half2float(v); }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float to_f<__nv_fp8_e4m3>(__nv_fp8_e4m3 v) { return static_cast<float>(v); }

template <typename TD> __device__ __forceinline__ void store_out(TD* p, float v, int trunc);
template <> __device__ __forceinline__ void store_out<float>(float* p, float v, int) { *p = v; }
template <> __device__ __forceinline__ void store_out<__half>(__half* p, float v, int) { *p = __float2half_rn(v); }
template <> __device__ __forceinline__ void store_out<__nv_bfloat16>(__nv_bfloat16* p, float v, int trunc)
{
    if (trunc) *reinterpret_cast<uint16_t*>(p) = static_cast<uint16_t>(__float_as_uint(v) >> 16);
    else *p = __float2bfloat16_rn(v);
}
template <typename TD> __device__ __forceinline__ float load_out(const TD* p) { return to_f<TD>(*p); }

struct SimtParams {
    const void* A;
    const void* B;
    const void* C;
    void* D;
    int64_t lda, ldb, ldc, ldd, sa, sb, sc, sd;
    int M, N, K;
    int trans_a, trans_b;
    float alpha, beta;
    int out_trunc;
};

// TM outputs per thread and dimension: 8 (128 x 128 tile) or 4 (64 x 64 tile), in TM/4 strips of 4
template <typename TA, typename TD, int TM>
__global__ void __launch_bounds__(THREADS, 2) simt_gemm_kernel(const SimtParams p)
{
    constexpr int BM = 16 * TM, BN = 16 * TM;   // 16 x 16 threads
    constexpr int LOADS = BM * BK / THREADS;    // elements of A (and of B) each thread stages per slab
    constexpr int STRIPS = TM / 4;
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Bs[2][BK][BN];

    const int tid = threadIdx.x;
    const int tx = tid & 15;          // m strip
    const int ty = tid >> 4;          // n strip
    const int m_blk = blockIdx.x * BM;
    const int n_blk = blockIdx.y * BN;
    const int b = blockIdx.z;
    const TA* A = static_cast<const TA*>(p.A) + static_cast<int64_t>(b) * p.sa;
    const TA* B = static_cast<const TA*>(p.B) + static_cast<int64_t>(b) * p.sb;

    // per-thread load coordinates: LOADS elements of A and of B per k-slab
    int a_m[LOADS], a_k[LOADS], b_n[LOADS], b_k[LOADS];
#pragma unroll
    for (int i = 0; i < LOADS; ++i) {
        const int idx = tid + i * THREADS;
        if (!p.trans_a) { a_m[i] = idx % BM; a_k[i] = idx / BM; }   // A[m + k*lda]: m contiguous
        else { a_m[i] = idx / BK; a_k[i] = idx % BK; }              // A[k + m*lda]: k contiguous
        if (p.trans_b) { b_n[i] = idx % BN; b_k[i] = idx / BN; }    // B[n + k*ldb]: n contiguous
        else { b_n[i] = idx / BK; b_k[i] = idx % BK; }              // B[k + n*ldb]: k contiguous
    }
    float ra[LOADS], rb[LOADS];
    auto load_slab = [&](int k0) {
#pragma unroll
        for (int i = 0; i < LOADS; ++i) {
            const int m = m_blk + a_m[i], k = k0 + a_k[i];
            float v = 0.f;
            if (m < p.M && k < p.K)
                v = to_f<TA>(p.trans_a ? A[k + static_cast<int64_t>(m) * p.lda] : A[m + static_cast<int64_t>(k) * p.lda]);
            ra[i] = v;
            const int n = n_blk + b_n[i], kb = k0 + b_k[i];
            float w = 0.f;
            if (n < p.N && kb < p.K)
                w = to_f<TA>(p.trans_b ? B[n + static_cast<int64_t>(kb) * p.ldb] : B[kb + static_cast<int64_t>(n) * p.ldb]);
            rb[i] = w;
        }
    };
    auto store_slab = [&](int buf) {
#pragma unroll
        for (int i = 0; i < LOADS; ++i) {
            As[buf][a_k[i]][a_m[i]] = ra[i];
            Bs[buf][b_k[i]][b_n[i]] = rb[i];
        }
    };

    float acc[TM][TM];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) acc[i][j] = 0.f;

    const int nslab = (p.K + BK - 1) / BK;
    if (nslab > 0) {
        load_slab(0);
        store_slab(0);
    }
    __syncthreads();
    for (int s = 0; s < nslab; ++s) {
        const int buf = s & 1;
        if (s + 1 < nslab) load_slab((s + 1) * BK);
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            float a[TM], bb[TM];
#pragma unroll
            for (int st = 0; st < STRIPS; ++st) {
                const float4 av = *reinterpret_cast<const float4*>(&As[buf][k][st * 64 + tx * 4]);
                const float4 bv = *reinterpret_cast<const float4*>(&Bs[buf][k][st * 64 + ty * 4]);
                a[4 * st] = av.x; a[4 * st + 1] = av.y; a[4 * st + 2] = av.z; a[4 * st + 3] = av.w;
                bb[4 * st] = bv.x; bb[4 * st + 1] = bv.y; bb[4 * st + 2] = bv.z; bb[4 * st + 3] = bv.w;
            }
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
        }
        if (s + 1 < nslab) store_slab(buf ^ 1);
        __syncthreads();
    }

    // epilogue: D = alpha*acc + beta*C (C not read when beta == 0)
    TD* D = static_cast<TD*>(p.D) + static_cast<int64_t>(b) * p.sd;
    const TD* C = p.C ? static_cast<const TD*>(p.C) + static_cast<int64_t>(b) * p.sc : nullptr;
    const bool use_c = (p.beta != 0.f) && (C != nullptr);
#pragma unroll
    for (int j = 0; j < TM; ++j) {
        const int n = n_blk + (j / 4) * 64 + ty * 4 + (j % 4);
        if (n >= p.N) continue;
#pragma unroll
        for (int i = 0; i < TM; ++i) {
            const int m = m_blk + (i / 4) * 64 + tx * 4 + (i % 4);
            if (m >= p.M) continue;
            float v = p.alpha * acc[i][j];
            if (use_c) v = fmaf(p.alpha, acc[i][j], p.beta * load_out<TD>(C + m + static_cast<int64_t>(n) * p.ldc));
            store_out<TD>(D + m + static_cast<int64_t>(n) * p.ldd, v, p.out_trunc);
        }
    }
}

template <typename TA, typename TD>
tl_status launch(const SimtLaunch& L, cudaStream_t s)
{
    SimtParams p;
    p.A = L.A; p.B = L.B; p.C = L.C; p.D = L.D;
    p.lda = L.lda; p.ldb = L.ldb; p.ldc = L.ldc; p.ldd = L.ldd;
    p.sa = L.sa; p.sb = L.sb; p.sc = L.sc; p.sd = L.sd;
    p.M = static_cast<int>(L.M); p.N = static_cast<int>(L.N); p.K = static_cast<int>(L.K);
    p.trans_a = L.trans_a; p.trans_b = L.trans_b;
    p.alpha = L.alpha; p.beta = L.beta;
    p.out_trunc = L.out_trunc;
    // 128 x 128 tiles, or 64 x 64 when the larger tiles would occupy fewer than half of the SMs
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    const int64_t big_tiles = ((L.M + 127) / 128) * ((L.N + 127) / 128) * L.batch;
    if (2 * big_tiles < sms) {
        dim3 grid(static_cast<unsigned>((L.M + 63) / 64), static_cast<unsigned>((L.N + 63) / 64),
                  static_cast<unsigned>(L.batch));
        simt_gemm_kernel<TA, TD, 4><<<grid, THREADS, 0, s>>>(p);
    } else {
        dim3 grid(static_cast<unsigned>((L.M + 127) / 128), static_cast<unsigned>((L.N + 127) / 128),
                  static_cast<unsigned>(L.batch));
        simt_gemm_kernel<TA, TD, 8><<<grid, THREADS, 0, s>>>(p);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "simt_gemm_kernel launch");
    return TL_SUCCESS;
}

template <typename TA>
tl_status launch_out(const SimtLaunch& L, cudaStream_t s)
{
    switch (L.out_dtype) {
    case TL_DTYPE_FP32: return launch<TA, float>(L, s);
    case TL_DTYPE_FP16: return launch<TA, __half>(L, s);
    case TL_DTYPE_BF16: return launch<TA, __nv_bfloat16>(L, s);
    default: return fail(TL_ERR_UNSUPPORTED, "SIMT kernel: unsupported output type");
    }
}

}  // namespace

tl_status simt_gemm_launch(const SimtLaunch& L, cudaStream_t s, int64_t* launches)
{
    if (L.M > 0x7fffffff || L.N > 0x7fffffff || L.K > 0x7fffffff || L.batch > 65535)
        return fail(TL_ERR_UNSUPPORTED, "SIMT kernel: dimension too large");
    if ((L.N + 63) / 64 > 65535) return fail(TL_ERR_UNSUPPORTED, "SIMT kernel: n too large");
    tl_status st;
    switch (L.a_dtype) {
    case TL_DTYPE_FP32: st = launch_out<float>(L, s); break;
    case TL_DTYPE_FP16: st = launch_out<__half>(L, s); break;
    case TL_DTYPE_BF16: st = launch_out<__nv_bfloat16>(L, s); break;
    case TL_DTYPE_FP8_E4M3: st = launch_out<__nv_fp8_e4m3>(L, s); break;
    default: return fail(TL_ERR_UNSUPPORTED, "SIMT kernel: unsupported input type");
    }
    if (st == TL_SUCCESS && launches) ++*launches;
    return st;
}

}  // namespace tl
