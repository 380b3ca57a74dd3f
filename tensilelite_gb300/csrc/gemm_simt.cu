// gemm_simt.cu -- CUDA-core GEMM (FP32 FMA pipes), any input type, fp32 accumulation.
//
// The plain-FP32 counterpart of TensileLite's sgemm path (the fp32 MFMA kernel,
// src/gemmMfmaKernelWriter.h:38-40) and the generic fallback for operands the TMA path cannot
// describe (leading dimensions that are not 16-byte multiples).
//
// Blackwell issues two fp32 FMAs per instruction (fma.rn.f32x2, __ffma2_rn): each thread keeps its
// TM x TN accumulators as float2 pairs along m, and one packed FMA multiplies a pair of A values by
// a B value held twice ({b, b}, formed in registers).  What bounds a CUDA-core GEMM on this SM is the
// shared-memory read path rather than the FMA pipes: a 16-byte shared load delivers 4 floats per
// thread over four cycles whatever the broadcast, so the SM reads at most 32 floats per cycle while
// its FMA pipes retire 128 FMAs.  A thread's outer-product step of TM x TN FMAs reads TM + TN
// floats, so the tiles per thread are as large as the registers allow: 16 x 8 (128 FMAs per 24
// floats, the shared path 75 % busy when the pipes are full).  B is stored once (not duplicated),
// which halves its shared reads at the cost of forming the {b, b} pairs in registers (issue slots
// are free: a packed FMA holds the pipe two cycles).
//
// Two shapes (chosen per problem on the host):
//   large  128 x 128 output tile, 128 threads, 16 x 8 outputs per thread, k in slabs of 8, two
//          CTAs per SM; tiles are rasterised in groups of 16 m-tiles so the tiles running together
//          share operand rows in L2;
//   small  64 x 32 output tile, 256 threads in 8 groups that each take an eighth of every 64-deep
//          k-slab (8 x 8 outputs per thread and group); the groups' partial tiles are summed in
//          group order through shared memory at the end.  For problems whose 128 x 128 tiles would
//          leave SMs idle (the reference's 480 x 512 x 512 case: 16 large tiles, 128 small ones),
//          one CTA per SM, slabs loaded two ahead.
// k-slabs are double-buffered in shared memory and prefetched into registers, with 4-element vector
// loads along whichever dimension is contiguous in memory; edge tiles are zero-filled on load and
// masked on store.  Results are deterministic (fixed summation order).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <type_traits>

#include "tl_internal.h"

namespace tl {
namespace tc {
bool pdl_enabled();   // programmatic dependent launch switch, shared with the tensor-core kernel
}
namespace {

template <typename T> __device__ __forceinline__ float to_f(T v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<__half>(__half v) { return __half2float(v); }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ float to_f<__nv_fp8_e4m3>(__nv_fp8_e4m3 v) { return static_cast<float>(v); }

// Four consecutive elements from a pointer aligned to 4 elements, widened to fp32.
template <typename T> __device__ __forceinline__ float4 load4(const T* p);
template <> __device__ __forceinline__ float4 load4<float>(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
template <> __device__ __forceinline__ float4 load4<__half>(const __half* p)
{
    const uint2 w = __ldg(reinterpret_cast<const uint2*>(p));
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&w.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&w.y));
    return make_float4(a.x, a.y, b.x, b.y);
}
template <> __device__ __forceinline__ float4 load4<__nv_bfloat16>(const __nv_bfloat16* p)
{
    const uint2 w = __ldg(reinterpret_cast<const uint2*>(p));
    return make_float4(__uint_as_float(w.x << 16), __uint_as_float(w.x & 0xffff0000u), __uint_as_float(w.y << 16),
                       __uint_as_float(w.y & 0xffff0000u));
}
template <> __device__ __forceinline__ float4 load4<__nv_fp8_e4m3>(const __nv_fp8_e4m3* p)
{
    return make_float4(to_f(p[0]), to_f(p[1]), to_f(p[2]), to_f(p[3]));
}

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
    int vec_a, vec_b;      // 4-element vector loads are aligned along the contiguous dimension
};

// Tile shape: BM x BN outputs, TM x TN per thread and k-group, KG k-groups, BKG k per group and slab,
// PD slabs loaded ahead into registers (1: the next slab's loads overlap one slab of FMAs; 2: two).
template <int BM_, int BN_, int TM_, int TN_, int KG_, int BKG_, int MINB_, int PD_>
struct Cfg {
    static constexpr int BM = BM_, BN = BN_, TM = TM_, TN = TN_, KG = KG_, BKG = BKG_, MINB = MINB_, PD = PD_;
    static constexpr int TX = BM / TM;           // threads along m in a group
    static constexpr int TY = BN / TN;           // threads along n
    static constexpr int GT = TX * TY;           // threads per k-group
    static constexpr int THREADS = GT * KG;
    static constexpr int BK = BKG * KG;          // k per slab
    static constexpr int SWM = TX * 4;           // width of one strip of 4 m-values per thread
    static constexpr int SWN = TY * 4;
    static constexpr int A_CHUNKS = BK * BM / 4 / THREADS;   // 4-element loads per thread and slab
    static constexpr int B_CHUNKS = BK * BN / 4 / THREADS;
    static constexpr int SMEM_FLOATS = 2 * BK * BM + 2 * BK * BN;
    static constexpr int RED_FLOATS = KG > 1 ? KG * BM * BN : 0;
    static constexpr size_t SMEM_BYTES = sizeof(float) * (SMEM_FLOATS > RED_FLOATS ? SMEM_FLOATS : RED_FLOATS);
    static_assert(TM % 4 == 0 && TN % 4 == 0, "per-thread tiles are strips of 4");
    static_assert(A_CHUNKS * THREADS * 4 == BK * BM && B_CHUNKS * THREADS * 4 == BK * BN, "whole slabs");
};
using CfgLarge = Cfg<128, 128, 16, 8, 1, 8, 2, 1>;
// one CTA per SM (it is used when tiles are fewer than SMs): up to 255 registers, 64-deep k-slabs,
// loads two slabs ahead (eight warps per SM cannot hide a DRAM round trip behind one slab)
using CfgSmall = Cfg<64, 32, 8, 8, 8, 8, 1, 2>;

constexpr int kRasterGroup = 16;   // m-tiles per raster group (tiles running together share B columns)

template <typename TA, typename TD, typename G>
__global__ void __launch_bounds__(G::THREADS, G::MINB) simt_gemm_kernel(const SimtParams p)
{
    constexpr int BM = G::BM, BN = G::BN, BK = G::BK, TM = G::TM, TN = G::TN;
    extern __shared__ __align__(16) float smem[];
    float* As = smem;                        // [2][BK][BM]      op(A)(m, k) at [k][m]
    float* Bs = smem + 2 * BK * BM;          // [2][BK][BN]      op(B)(k, n) at [k][n]

    const int tid = threadIdx.x;
    const int grp = tid / G::GT;             // k-group
    const int gtid = tid % G::GT;
    const int tx = gtid % G::TX;
    const int ty = gtid / G::TX;
    // raster: blocks walk groups of kRasterGroup m-tiles, m fastest, so the tiles running together
    // share their B columns and a band of A rows in L2
    const int tiles_m = (p.M + BM - 1) / BM, tiles_n = (p.N + BN - 1) / BN;
    const int lin = blockIdx.x;
    const int gsz = kRasterGroup * tiles_n;
    const int first_m = (lin / gsz) * kRasterGroup;
    const int gw = min(kRasterGroup, tiles_m - first_m);
    const int m_blk = (first_m + (lin % gsz) % gw) * BM;
    const int n_blk = ((lin % gsz) / gw) * BN;
    const int b = blockIdx.z;
    // Launched as a programmatic dependent: wait for the previous grid in the stream to complete
    // (its writes visible) before the first global access, then let the next grid get scheduled.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const TA* A = static_cast<const TA*>(p.A) + static_cast<int64_t>(b) * p.sa;
    const TA* B = static_cast<const TA*>(p.B) + static_cast<int64_t>(b) * p.sb;

    // ---- global -> registers (PD slabs ahead) -> shared; register set r holds the slabs s with
    // s % PD == r (indexes are compile-time constants after inlining)
    float4 ra[G::PD][G::A_CHUNKS], rb[G::PD][G::B_CHUNKS];
    auto load_slab = [&](auto rset, int k0) {
        constexpr int r = decltype(rset)::value;
#pragma unroll
        for (int c = 0; c < G::A_CHUNKS; ++c) {
            const int idx = tid + c * G::THREADS;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (!p.trans_a) {                // A[m + k*lda]: 4 consecutive m of one k
                const int m = m_blk + (idx % (BM / 4)) * 4, k = k0 + idx / (BM / 4);
                const TA* src = A + m + static_cast<int64_t>(k) * p.lda;
                if (k < p.K) {
                    if (p.vec_a && m + 3 < p.M) v = load4<TA>(src);
                    else {
                        if (m < p.M) v.x = to_f<TA>(src[0]);
                        if (m + 1 < p.M) v.y = to_f<TA>(src[1]);
                        if (m + 2 < p.M) v.z = to_f<TA>(src[2]);
                        if (m + 3 < p.M) v.w = to_f<TA>(src[3]);
                    }
                }
            } else {                         // A[k + m*lda]: 4 consecutive k of one m
                const int m = m_blk + idx % BM, k = k0 + (idx / BM) * 4;
                const TA* src = A + k + static_cast<int64_t>(m) * p.lda;
                if (m < p.M) {
                    if (p.vec_a && k + 3 < p.K) v = load4<TA>(src);
                    else {
                        if (k < p.K) v.x = to_f<TA>(src[0]);
                        if (k + 1 < p.K) v.y = to_f<TA>(src[1]);
                        if (k + 2 < p.K) v.z = to_f<TA>(src[2]);
                        if (k + 3 < p.K) v.w = to_f<TA>(src[3]);
                    }
                }
            }
            ra[r][c] = v;
        }
#pragma unroll
        for (int c = 0; c < G::B_CHUNKS; ++c) {
            const int idx = tid + c * G::THREADS;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (p.trans_b) {                 // B[n + k*ldb]: 4 consecutive n of one k
                const int n = n_blk + (idx % (BN / 4)) * 4, k = k0 + idx / (BN / 4);
                const TA* src = B + n + static_cast<int64_t>(k) * p.ldb;
                if (k < p.K) {
                    if (p.vec_b && n + 3 < p.N) v = load4<TA>(src);
                    else {
                        if (n < p.N) v.x = to_f<TA>(src[0]);
                        if (n + 1 < p.N) v.y = to_f<TA>(src[1]);
                        if (n + 2 < p.N) v.z = to_f<TA>(src[2]);
                        if (n + 3 < p.N) v.w = to_f<TA>(src[3]);
                    }
                }
            } else {                         // B[k + n*ldb]: 4 consecutive k of one n
                const int n = n_blk + idx % BN, k = k0 + (idx / BN) * 4;
                const TA* src = B + k + static_cast<int64_t>(n) * p.ldb;
                if (n < p.N) {
                    if (p.vec_b && k + 3 < p.K) v = load4<TA>(src);
                    else {
                        if (k < p.K) v.x = to_f<TA>(src[0]);
                        if (k + 1 < p.K) v.y = to_f<TA>(src[1]);
                        if (k + 2 < p.K) v.z = to_f<TA>(src[2]);
                        if (k + 3 < p.K) v.w = to_f<TA>(src[3]);
                    }
                }
            }
            rb[r][c] = v;
        }
    };
    auto store_slab = [&](auto rset, int buf) {
        constexpr int r = decltype(rset)::value;
        float* as = As + buf * BK * BM;
        float* bs = Bs + buf * BK * BN;
#pragma unroll
        for (int c = 0; c < G::A_CHUNKS; ++c) {
            const int idx = tid + c * G::THREADS;
            if (!p.trans_a) {
                const int m = (idx % (BM / 4)) * 4, k = idx / (BM / 4);
                *reinterpret_cast<float4*>(as + k * BM + m) = ra[r][c];
            } else {
                const int m = idx % BM, k = (idx / BM) * 4;
                as[(k + 0) * BM + m] = ra[r][c].x;
                as[(k + 1) * BM + m] = ra[r][c].y;
                as[(k + 2) * BM + m] = ra[r][c].z;
                as[(k + 3) * BM + m] = ra[r][c].w;
            }
        }
#pragma unroll
        for (int c = 0; c < G::B_CHUNKS; ++c) {
            const int idx = tid + c * G::THREADS;
            if (p.trans_b) {
                const int n = (idx % (BN / 4)) * 4, k = idx / (BN / 4);
                *reinterpret_cast<float4*>(bs + k * BN + n) = rb[r][c];
            } else {
                const int n = idx % BN, k = (idx / BN) * 4;
                const float4 q = rb[r][c];
                bs[(k + 0) * BN + n] = q.x;
                bs[(k + 1) * BN + n] = q.y;
                bs[(k + 2) * BN + n] = q.z;
                bs[(k + 3) * BN + n] = q.w;
            }
        }
    };

    // acc[i][j] holds outputs (m_{2i}, n_j) and (m_{2i+1}, n_j); m_r = (r/4)*SWM + tx*4 + r%4,
    // n_j = (j/4)*SWN + ty*4 + j%4
    float2 acc[TM / 2][TN];
#pragma unroll
    for (int i = 0; i < TM / 2; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = make_float2(0.f, 0.f);

    auto compute_slab = [&](int buf) {
        const float* as = As + buf * BK * BM + grp * G::BKG * BM;
        const float* bs = Bs + buf * BK * BN + grp * G::BKG * BN;
#pragma unroll
        for (int kk = 0; kk < G::BKG; ++kk) {
            float2 a[TM / 2], bd[TN];
#pragma unroll
            for (int st = 0; st < TM / 4; ++st) {
                const float4 v = *reinterpret_cast<const float4*>(as + kk * BM + st * G::SWM + tx * 4);
                a[2 * st] = make_float2(v.x, v.y);
                a[2 * st + 1] = make_float2(v.z, v.w);
            }
#pragma unroll
            for (int st = 0; st < TN / 4; ++st) {
                const float4 v = *reinterpret_cast<const float4*>(bs + kk * BN + st * G::SWN + ty * 4);
                bd[4 * st + 0] = make_float2(v.x, v.x);
                bd[4 * st + 1] = make_float2(v.y, v.y);
                bd[4 * st + 2] = make_float2(v.z, v.z);
                bd[4 * st + 3] = make_float2(v.w, v.w);
            }
#pragma unroll
            for (int i = 0; i < TM / 2; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = __ffma2_rn(a[i], bd[j], acc[i][j]);
        }
    };
    using R0 = std::integral_constant<int, 0>;
    using R1 = std::integral_constant<int, G::PD - 1>;
    const int nslab = (p.K + BK - 1) / BK;
    if (nslab > 0) {
        load_slab(R0{}, 0);
        store_slab(R0{}, 0);
    }
    if constexpr (G::PD == 1) {
        __syncthreads();
        for (int s = 0; s < nslab; ++s) {
            const int buf = s & 1;
            if (s + 1 < nslab) load_slab(R0{}, (s + 1) * BK);
            compute_slab(buf);
            if (s + 1 < nslab) store_slab(R0{}, buf ^ 1);
            __syncthreads();
        }
    } else {
        // slab s is computed from shared buffer s & 1 while slab s + 2 is loaded into register set
        // s & 1 (slab s went from that set to shared memory a step earlier) and slab s + 1 moves
        // from register set (s + 1) & 1 into the other shared buffer
        if (nslab > 1) load_slab(R1{}, BK);
        __syncthreads();
        auto step = [&](auto rset, int s) {
            constexpr int r = decltype(rset)::value;
            using RN = std::integral_constant<int, r ^ 1>;
            if (s + 2 < nslab) load_slab(rset, (s + 2) * BK);
            compute_slab(r);
            if (s + 1 < nslab) store_slab(RN{}, r ^ 1);
            __syncthreads();
        };
        for (int s = 0; s < nslab; s += 2) {
            step(R0{}, s);
            if (s + 1 < nslab) step(R1{}, s + 1);
        }
    }

    // ---- epilogue: D = alpha*acc + beta*C (C not read when beta == 0)
    TD* D = static_cast<TD*>(p.D) + static_cast<int64_t>(b) * p.sd;
    const TD* C = p.C ? static_cast<const TD*>(p.C) + static_cast<int64_t>(b) * p.sc : nullptr;
    const bool use_c = (p.beta != 0.f) && (C != nullptr);
    auto finish = [&](int m, int n, float v) {
        float o = p.alpha * v;
        if (use_c) o = fmaf(p.alpha, v, p.beta * load_out<TD>(C + m + static_cast<int64_t>(n) * p.ldc));
        store_out<TD>(D + m + static_cast<int64_t>(n) * p.ldd, o, p.out_trunc);
    };
    if constexpr (G::KG == 1) {
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = n_blk + (j / 4) * G::SWN + ty * 4 + (j % 4);
            if (n >= p.N) continue;
#pragma unroll
            for (int i = 0; i < TM / 2; ++i) {
                const int m = m_blk + ((2 * i) / 4) * G::SWM + tx * 4 + (2 * i) % 4;
                if (m < p.M) finish(m, n, acc[i][j].x);
                if (m + 1 < p.M) finish(m + 1, n, acc[i][j].y);
            }
        }
    } else {
        // the k-groups' partial tiles, [group][n][m], summed in group order
        float* red = smem;                   // the slab buffers are free after the last sync
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int n = (j / 4) * G::SWN + ty * 4 + (j % 4);
#pragma unroll
            for (int i = 0; i < TM / 2; ++i) {
                const int m = ((2 * i) / 4) * G::SWM + tx * 4 + (2 * i) % 4;
                *reinterpret_cast<float2*>(red + (grp * BN + n) * BM + m) = acc[i][j];
            }
        }
        __syncthreads();
        for (int e = tid; e < BM * BN; e += G::THREADS) {
            const int m = e % BM, n = e / BM;
            float v = red[n * BM + m];
#pragma unroll
            for (int g = 1; g < G::KG; ++g) v += red[(g * BN + n) * BM + m];
            if (m_blk + m < p.M && n_blk + n < p.N) finish(m_blk + m, n_blk + n, v);
        }
    }
}

template <typename TA, typename TD, typename G>
tl_status launch_cfg(const SimtParams& p, int64_t M, int64_t N, int64_t batch, cudaStream_t s)
{
    auto kern = simt_gemm_kernel<TA, TD, G>;
    if constexpr (G::SMEM_BYTES > 48 * 1024) {
        static const cudaError_t attr =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(G::SMEM_BYTES));
        if (attr != cudaSuccess) return cuda_fail(attr, "cudaFuncSetAttribute(simt_gemm_kernel)");
    }
    const int64_t tiles = ((M + G::BM - 1) / G::BM) * ((N + G::BN - 1) / G::BN);
    if (tiles > 0x7fffffff) return fail(TL_ERR_UNSUPPORTED, "SIMT kernel: too many tiles");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(tiles), 1, static_cast<unsigned>(batch));
    cfg.blockDim = dim3(G::THREADS, 1, 1);
    cfg.dynamicSmemBytes = G::SMEM_BYTES;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    if (tc::pdl_enabled()) {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, p);
    if (e != cudaSuccess) return cuda_fail(e, "cudaLaunchKernelEx(simt_gemm_kernel)");
    return TL_SUCCESS;
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
    // vector loads need the 4-element groups aligned: base, leading dimension and batch stride
    const uintptr_t vb = 4 * sizeof(TA);
    p.vec_a = ((reinterpret_cast<uintptr_t>(L.A) % vb) == 0 && L.lda % 4 == 0 && (L.batch == 1 || L.sa % 4 == 0)) ? 1 : 0;
    p.vec_b = ((reinterpret_cast<uintptr_t>(L.B) % vb) == 0 && L.ldb % 4 == 0 && (L.batch == 1 || L.sb % 4 == 0)) ? 1 : 0;
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    // 128 x 128 tiles, or the k-grouped 64 x 32 tiles when the large ones would leave SMs idle
    const int64_t big_tiles = ((L.M + 127) / 128) * ((L.N + 127) / 128) * L.batch;
    if (big_tiles < sms) return launch_cfg<TA, TD, CfgSmall>(p, L.M, L.N, L.batch, s);
    return launch_cfg<TA, TD, CfgLarge>(p, L.M, L.N, L.batch, s);
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
