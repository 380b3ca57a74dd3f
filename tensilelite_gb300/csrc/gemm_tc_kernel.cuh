// The tcgen05 GEMM kernel template and its launch templates, shared by the translation unit with the
// host code (gemm_tc.cu) and the instance units the build generates (one per operand kind, cluster
// size and epilogue variant, compiled in parallel).  See gemm_tc.cu for the design notes.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include "ptx.cuh"
#include "tl_internal.h"

namespace tl {
namespace tc {


struct TcKernelParams {
    CUtensorMap tmN[3], tmM[3];   // split-precision pieces 0..2 (piece 0 = the operand itself)
    CUtensorMap tmD;              // the output, boxes of 128 bytes x 32 rows (tma_store)
    int tma_store;                // whole tiles leave through shared memory and TMA stores
    int direct_last;              // a CTA's last tile (beta == 0) leaves through direct stores
    // fused epilogue (kernels instantiated with EPI): D = act(alpha*acc + beta*C + bias[m]), and
    // max |D| into *epi_amax
    const void* epi_bias;
    float* epi_amax;
    float epi_dscale;             // fp8 outputs: values are multiplied by this before the E4M3 rounding
    int epi_bias_dtype;
    int epi_act;
    int epi_on;
    int par_reduce;               // every split unit runs in the first round: the splits of a tile
                                  // wait for each other and reduce one share of it each
    const TcGroupEntry* group;
    const int4* group_units;       // per work unit: {problem, tile row, tile column, k-blocks}
    void* D;
    const void* C;
    int64_t ldd, ldc, stride_d, stride_c;
    int M, N, K, batch;
    float alpha, beta;
    int bm, stages, split_k, raster;
    int tile_rows;                // n rows per tile: 128 (one CTA) or 256 (CTA pair)
    int nterms;                   // tensor-core products per k-block (1, or 3 / 6 for the fp32 split)
    uint8_t term_n[8], term_m[8]; // piece of B / of A used by each product (the last is A0*B0)
    int promote_kb;               // >0: the A0*B0 product restarts its TMEM chain every promote_kb
                                  // k-blocks; the epilogue adds each chain into fp32 registers
    int tiles_m, tiles_n;
    int narrow;                   // work units, tiles and split k-block products fit 32 bits
    int64_t total_work;
    int64_t split_units;          // work units below this are k-slices of the first split_tiles tiles
    int64_t split_tiles;          // tiles split along k; the rest are whole
    int tail_split;               // k slices of each split tile (balanced: the workspace slab stride)
    // balanced split (bal_kb > 0): the split tiles' bal_kb k-blocks are cut into bal_workers equal
    // contiguous ranges, one per worker; unit w < 2 * bal_stride is piece w / bal_stride (a range
    // spans at most two tiles) of worker w % bal_stride
    int64_t bal_kb;
    int bal_workers;
    int bal_stride;
    int num_kb;
    int kb_elems;          // k elements per k-block (one 128-byte row)
    uint32_t idesc;
    uint32_t n_lbo, m_lbo, n_kstep, m_kstep;
    int n_mn_major, m_mn_major;
    int out_trunc;
    float* ws;
    int* counters;
    int* err;
    unsigned long long timeout_ns;
    int debug_skip_loads;         // TL_DEBUG_SKIP_LOADS: the producer issues no copies (timeout-path test)
    unsigned long long* trace;    // device timeline, TL_TRACE_SLOTS words per CTA, or null
    int out_t;                    // D and C are the transpose of the kernel's output: element (m, n)
                                  // at n + m * ld (an NN problem run as its transposed TT product)
};

// Timeline stamp of event `slot` for this CTA (tl_set_trace): the SM cycle counter.
__device__ __forceinline__ void trace_mark(const TcKernelParams& p, int slot)
{
    if (p.trace != nullptr) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%clock64;" : "=l"(t) :: "memory");
        p.trace[static_cast<size_t>(blockIdx.x) * TL_TRACE_SLOTS + slot] = t;
    }
}
__device__ __forceinline__ void trace_put(const TcKernelParams& p, int slot, unsigned long long v)
{
    if (p.trace != nullptr) p.trace[static_cast<size_t>(blockIdx.x) * TL_TRACE_SLOTS + slot] = v;
}
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t) :: "memory");
    return t;
}

struct TileJob {
    const void* tmN;
    const void* tmM;
    const CUtensorMap* tmD;       // the output for TMA stores, or null
    void* D;
    const void* C;
    int64_t ldd, ldc;
    int M, N;
    float alpha, beta;
    int b, n0, m0;
    int kb0, kb1;
    int split, nsplit;            // this unit's k split and the tile's number of splits
    int out_t;                    // transposed output (TcKernelParams::out_t)
    int64_t tile;
    int64_t slot;                 // split tiles: index of the tile's workspace slabs and counter
};

// Grouped launches: the unit-table entry of work unit w (a zero entry past the end or without a group).
__device__ __forceinline__ int4 load_unit(const TcKernelParams& p, int64_t w)
{
    if (p.group == nullptr || w >= p.total_work) return make_int4(0, 0, 0, 0);
    return __ldg(p.group_units + w);
}

__device__ __forceinline__ void get_job(const TcKernelParams& p, int64_t w, const int4& u, TileJob& j)
{
    if (p.group == nullptr) {
        int64_t tile;
        int split, nsplit;
        int kb0, kb1;
        if (p.bal_kb > 0 && w < 2 * static_cast<int64_t>(p.bal_stride)) {
            // balanced split: worker `wk` owns k-blocks [s0, s1) of the split tiles laid end to end;
            // piece 0 is the part in its first tile, piece 1 the rest (possibly empty)
            const int64_t wk = w % p.bal_stride, piece = w / p.bal_stride;
            const int64_t R = p.bal_kb, Wb = p.bal_workers, nkb = p.num_kb;
            int64_t a = 0, e = 0;
            if (wk < Wb) {
                const int64_t s0 = wk * R / Wb, s1 = (wk + 1) * R / Wb;
                const int64_t cut = min(s1, (s0 / nkb + 1) * nkb);
                a = piece == 0 ? s0 : cut;
                e = piece == 0 ? cut : s1;
            }
            if (a >= e) {
                tile = 0;                    // empty unit: every role skips it
                kb0 = kb1 = 0;
                split = 0;
                nsplit = 1;
            } else {
                tile = a / nkb;
                kb0 = static_cast<int>(a - tile * nkb);
                kb1 = static_cast<int>(e - tile * nkb);
                // the workers covering this tile: the one holding its first and its last k-block
                const int64_t first = ((tile * nkb + 1) * Wb - 1) / R;
                const int64_t last = (((tile + 1) * nkb) * Wb - 1) / R;
                nsplit = static_cast<int>(last - first + 1);
                split = static_cast<int>(wk - first);
            }
        } else if (w < p.split_units) {
            // split tiles come first, so the last arriver's reduction overlaps later whole tiles
            nsplit = p.tail_split;
            if (p.narrow) {
                const uint32_t uw = static_cast<uint32_t>(w), ts = static_cast<uint32_t>(nsplit);
                const uint32_t q = uw / ts, nkb = static_cast<uint32_t>(p.num_kb);
                tile = q;
                split = static_cast<int>(uw - q * ts);
                kb0 = static_cast<int>((static_cast<uint32_t>(split) * nkb) / ts);
                kb1 = static_cast<int>((static_cast<uint32_t>(split + 1) * nkb) / ts);
            } else {
                tile = w / p.tail_split;
                split = static_cast<int>(w % p.tail_split);
                kb0 = static_cast<int>((static_cast<int64_t>(split) * p.num_kb) / nsplit);
                kb1 = static_cast<int>((static_cast<int64_t>(split + 1) * p.num_kb) / nsplit);
            }
        } else {
            tile = p.split_tiles + (w - p.split_units);
            split = 0;
            nsplit = 1;
            kb0 = 0;
            kb1 = p.num_kb;
        }
        int b, in, jm;
        if (p.narrow) {
            // every tile index fits 32 bits (host-checked): 32-bit divisions are several times
            // shorter than 64-bit ones, and this decode sits between the launch and the first load
            const uint32_t ut = static_cast<uint32_t>(tile);
            const uint32_t tpb = static_cast<uint32_t>(p.tiles_m) * static_cast<uint32_t>(p.tiles_n);
            const uint32_t ub = ut / tpb;
            const uint32_t t = ut - ub * tpb;
            b = static_cast<int>(ub);
            if (p.raster > 0) {
                const uint32_t group_tiles = static_cast<uint32_t>(p.raster) * static_cast<uint32_t>(p.tiles_m);
                const uint32_t g = t / group_tiles;
                const int first_n = static_cast<int>(g * static_cast<uint32_t>(p.raster));
                const uint32_t gsize = static_cast<uint32_t>(min(p.raster, p.tiles_n - first_n));
                const uint32_t r = t - g * group_tiles;
                const uint32_t rq = r / gsize;
                in = first_n + static_cast<int>(r - rq * gsize);
                jm = static_cast<int>(rq);
            } else {
                const uint32_t q = t / static_cast<uint32_t>(p.tiles_m);
                in = static_cast<int>(q);
                jm = static_cast<int>(t - q * static_cast<uint32_t>(p.tiles_m));
            }
        } else {
            const int64_t tpb = static_cast<int64_t>(p.tiles_m) * p.tiles_n;
            b = static_cast<int>(tile / tpb);
            const int64_t t = tile % tpb;
            if (p.raster > 0) {
                const int64_t group_tiles = static_cast<int64_t>(p.raster) * p.tiles_m;
                const int64_t g = t / group_tiles;
                const int first_n = static_cast<int>(g * p.raster);
                const int gsize = min(p.raster, p.tiles_n - first_n);
                const int64_t r = t % group_tiles;
                in = first_n + static_cast<int>(r % gsize);
                jm = static_cast<int>(r / gsize);
            } else {
                in = static_cast<int>(t / p.tiles_m);
                jm = static_cast<int>(t % p.tiles_m);
            }
        }
        j.tmN = &p.tmN[0];
        j.tmM = &p.tmM[0];
        j.tmD = p.tma_store ? &p.tmD : nullptr;
        j.D = static_cast<char*>(p.D);
        j.C = p.C;
        j.ldd = p.ldd;
        j.ldc = p.ldc;
        j.M = p.M;
        j.N = p.N;
        j.alpha = p.alpha;
        j.beta = p.beta;
        j.b = b;
        j.n0 = in * p.tile_rows;
        j.m0 = jm * p.bm;
        j.kb0 = kb0;
        j.kb1 = kb1;
        j.split = split;
        j.nsplit = nsplit;
        j.out_t = p.out_t;
        j.tile = tile;
        j.slot = tile;                 // split tiles are 0 .. split_tiles-1
    } else {
        // grouped: the unit's problem and tile come from the plan's unit table (loaded ahead by
        // the caller); only the epilogue reads the problem's entry
        const TcGroupEntry& e = p.group[u.x];
        j.tmN = &e.tmN;
        j.tmM = &e.tmM;
        j.tmD = e.tma_store ? &e.tmD : nullptr;
        j.D = e.D;
        j.C = e.C;
        j.ldd = e.ldd;
        j.ldc = e.ldc;
        j.M = e.M;
        j.N = e.N;
        j.alpha = e.alpha;
        j.beta = e.beta;
        j.b = 0;
        j.n0 = u.y * p.tile_rows;
        j.m0 = u.z * p.bm;
        j.kb0 = 0;
        j.kb1 = u.w;
        j.split = 0;
        j.nsplit = 1;
        j.out_t = 0;
        j.tile = w;
        j.slot = 0;
    }
}

__device__ __forceinline__ void record_error(const TcKernelParams& p, volatile int* abort_flag, int code)
{
    *abort_flag = 1;
    atomicOr(p.err, code);
}

// ---- output conversion ------------------------------------------------------------------------------
template <typename TD> struct Out;
template <> struct Out<float> {
    __device__ static __forceinline__ float load(const void* base, int64_t idx)
    { return __ldg(static_cast<const float*>(base) + idx); }
    __device__ static __forceinline__ void store(void* base, int64_t idx, float v, int)
    { static_cast<float*>(base)[idx] = v; }
    static constexpr int kBytes = 4;
};
template <> struct Out<__half> {
    __device__ static __forceinline__ float load(const void* base, int64_t idx)
    { return __half2float(static_cast<const __half*>(base)[idx]); }
    __device__ static __forceinline__ void store(void* base, int64_t idx, float v, int)
    { static_cast<__half*>(base)[idx] = __float2half_rn(v); }
    static constexpr int kBytes = 2;
};
template <> struct Out<__nv_bfloat16> {
    __device__ static __forceinline__ float load(const void* base, int64_t idx)
    { return __bfloat162float(static_cast<const __nv_bfloat16*>(base)[idx]); }
    __device__ static __forceinline__ void store(void* base, int64_t idx, float v, int trunc)
    {
        if (trunc) static_cast<uint16_t*>(base)[idx] = static_cast<uint16_t>(__float_as_uint(v) >> 16);
        else static_cast<__nv_bfloat16*>(base)[idx] = __float2bfloat16_rn(v);
    }
    static constexpr int kBytes = 2;
};

// E4M3 outputs (fused-epilogue kernels; beta must be 0): round to nearest even, saturating to +-448.
template <> struct Out<__nv_fp8_e4m3> {
    __device__ static __forceinline__ float load(const void* base, int64_t idx)
    {
        return __half2float(__half(__nv_cvt_fp8_to_halfraw(static_cast<const __nv_fp8_storage_t*>(base)[idx], __NV_E4M3)));
    }
    __device__ static __forceinline__ void store(void* base, int64_t idx, float v, int)
    { static_cast<__nv_fp8_storage_t*>(base)[idx] = __nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3); }
    static constexpr int kBytes = 1;
};

// Four values as four E4M3 bytes in one word (first value in the low byte).
__device__ __forceinline__ uint32_t pack4_e4m3(float a, float b, float c, float d)
{
    const uint32_t lo = __nv_cvt_float2_to_fp8x2(make_float2(a, b), __NV_SATFINITE, __NV_E4M3);
    const uint32_t hi = __nv_cvt_float2_to_fp8x2(make_float2(c, d), __NV_SATFINITE, __NV_E4M3);
    return (lo & 0xffffu) | (hi << 16);
}

// The quantisation scale of fp8 outputs (applied after the epilogue function and the amax).
template <typename TD>
__device__ __forceinline__ float out_scale(const TcKernelParams& p, float o)
{
    if constexpr (sizeof(TD) == 1) return o * p.epi_dscale;
    else return o;
}

__device__ __forceinline__ uint32_t pack2(float a, float b, int is_half, int trunc)
{
    if (is_half) {
        __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t*>(&h);
    }
    if (trunc) return (__float_as_uint(a) >> 16) | (__float_as_uint(b) & 0xffff0000u);
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ void unpack2(uint32_t w, int is_half, float& a, float& b)
{
    if (is_half) {
        __half2 h = *reinterpret_cast<__half2*>(&w);
        float2 f = __half22float2(h);
        a = f.x;
        b = f.y;
    } else {
        a = __uint_as_float(w << 16);
        b = __uint_as_float(w & 0xffff0000u);
    }
}

// Fused epilogue of one output value at row m: + bias[m], activation (1 relu, 2 gelu with the tanh
// approximation, 3 silu), and the running max |value| of this thread over the stored values.
__device__ __forceinline__ float epi_fn(const TcKernelParams& p, int m, bool stored, float o, float& amax)
{
    if (p.epi_bias != nullptr && stored) {
        if (p.epi_bias_dtype == TL_DTYPE_FP32) o += __ldg(static_cast<const float*>(p.epi_bias) + m);
        else if (p.epi_bias_dtype == TL_DTYPE_FP16) o += __half2float(static_cast<const __half*>(p.epi_bias)[m]);
        else o += __bfloat162float(static_cast<const __nv_bfloat16*>(p.epi_bias)[m]);
    }
    if (p.epi_act == 1) {
        o = fmaxf(o, 0.0f);
    } else if (p.epi_act == 2) {
        const float u = 0.7978845608028654f * fmaf(0.044715f * o * o, o, o);
        o = 0.5f * o * (1.0f + tanhf(u));
    } else if (p.epi_act == 3) {
        o = o / (1.0f + expf(-o));
    }
    if (stored) amax = fmaxf(amax, fabsf(o));
    return o;
}

// Finish 32 consecutive outputs m..m+31 of column n: v = alpha*acc + beta*C (then the fused
// epilogue when EPI), convert, store.
template <typename TD, bool EPI>
__device__ __forceinline__ void store_chunk(const TcKernelParams& p, float& amax, const TileJob& j, int64_t base_c,
                                           int64_t base_d, int m, float (&acc)[32], int trunc)
{
    const bool full = (m + 32 <= j.M);
    const bool use_c = (j.beta != 0.0f) && (j.C != nullptr);
    char* dptr = static_cast<char*>(j.D) + (base_d + m) * Out<TD>::kBytes;
    const char* cptr = use_c ? static_cast<const char*>(j.C) + (base_c + m) * Out<TD>::kBytes : nullptr;
    const bool vec = full && !j.out_t && ((reinterpret_cast<uintptr_t>(dptr) & 15) == 0) &&
                     (!use_c || (reinterpret_cast<uintptr_t>(cptr) & 15) == 0);
    if (vec) {
        if constexpr (sizeof(TD) == 4) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float4 c4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (use_c) c4 = __ldg(reinterpret_cast<const float4*>(cptr) + q);
                float4 o;
                if (use_c) {
                    o.x = fmaf(j.alpha, acc[4 * q + 0], j.beta * c4.x);
                    o.y = fmaf(j.alpha, acc[4 * q + 1], j.beta * c4.y);
                    o.z = fmaf(j.alpha, acc[4 * q + 2], j.beta * c4.z);
                    o.w = fmaf(j.alpha, acc[4 * q + 3], j.beta * c4.w);
                } else {
                    o.x = j.alpha * acc[4 * q + 0];
                    o.y = j.alpha * acc[4 * q + 1];
                    o.z = j.alpha * acc[4 * q + 2];
                    o.w = j.alpha * acc[4 * q + 3];
                }
                if constexpr (EPI) {
                    o.x = epi_fn(p, m + 4 * q + 0, true, o.x, amax);
                    o.y = epi_fn(p, m + 4 * q + 1, true, o.y, amax);
                    o.z = epi_fn(p, m + 4 * q + 2, true, o.z, amax);
                    o.w = epi_fn(p, m + 4 * q + 3, true, o.w, amax);
                }
                reinterpret_cast<float4*>(dptr)[q] = o;
            }
        } else if constexpr (sizeof(TD) == 1) {
            // E4M3: 32 outputs in two 16-byte stores (no C: fp8 outputs take beta == 0)
            uint32_t ow[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float o[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    o[t] = j.alpha * acc[4 * q + t];
                    if constexpr (EPI) o[t] = epi_fn(p, m + 4 * q + t, true, o[t], amax);
                    o[t] = out_scale<TD>(p, o[t]);
                }
                ow[q] = pack4_e4m3(o[0], o[1], o[2], o[3]);
            }
            reinterpret_cast<uint4*>(dptr)[0] = make_uint4(ow[0], ow[1], ow[2], ow[3]);
            reinterpret_cast<uint4*>(dptr)[1] = make_uint4(ow[4], ow[5], ow[6], ow[7]);
        } else {
            constexpr int is_half = std::is_same<TD, __half>::value ? 1 : 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint4 cw = make_uint4(0, 0, 0, 0);
                if (use_c) cw = __ldg(reinterpret_cast<const uint4*>(cptr) + q);
                uint32_t cws[4] = {cw.x, cw.y, cw.z, cw.w};
                uint32_t ow[4];
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    float c0 = 0.f, c1 = 0.f;
                    if (use_c) unpack2(cws[h], is_half, c0, c1);
                    const float a0 = acc[8 * q + 2 * h], a1 = acc[8 * q + 2 * h + 1];
                    float o0 = use_c ? fmaf(j.alpha, a0, j.beta * c0) : j.alpha * a0;
                    float o1 = use_c ? fmaf(j.alpha, a1, j.beta * c1) : j.alpha * a1;
                    if constexpr (EPI) {
                        o0 = epi_fn(p, m + 8 * q + 2 * h, true, o0, amax);
                        o1 = epi_fn(p, m + 8 * q + 2 * h + 1, true, o1, amax);
                    }
                    ow[h] = pack2(o0, o1, is_half, trunc);
                }
                reinterpret_cast<uint4*>(dptr)[q] = make_uint4(ow[0], ow[1], ow[2], ow[3]);
            }
        }
    } else {
        // element m + i at (m + i) * step: 1, or ld for a transposed output (a warp's 32 rows then
        // make one coalesced access per element)
        // C in groups of sixteen, each group read before its D is written: the loads of a group
        // overlap (a store may alias a later load, so none is moved above one), and D may be C itself
        const int64_t dstep = j.out_t ? j.ldd : 1, cstep = j.out_t ? j.ldc : 1;
#pragma unroll
        for (int i0 = 0; i0 < 32; i0 += 16) {
            float cv[16];
#pragma unroll
            for (int t = 0; t < 16; ++t)
                cv[t] = (use_c && m + i0 + t < j.M) ? Out<TD>::load(j.C, base_c + (m + i0 + t) * cstep) : 0.f;
#pragma unroll
            for (int t = 0; t < 16; ++t) {
                const int i = i0 + t;
                if (m + i < j.M) {
                    float o = use_c ? fmaf(j.alpha, acc[i], j.beta * cv[t]) : j.alpha * acc[i];
                    if constexpr (EPI) o = epi_fn(p, m + i, true, o, amax);
                    Out<TD>::store(j.D, base_d + (m + i) * dstep, out_scale<TD>(p, o), trunc);
                }
            }
        }
    }
}

// Split-k completion, run by the four epilogue warps after this split parked its partial tile in
// the workspace (layout [32-column chunk][column][row], so every warp access is one 128-byte line): the last split of a tile to arrive (per-tile counter) sums every split's partial
// in split order -- so the result does not depend on which CTA finished last -- and runs the
// epilogue.  The counter is reset for the next launch.  Every thread passes the same three named
// barriers whether or not it has work, so a warp that gave up on a wait cannot strand the others.
template <typename TD, bool EPI>
__device__ __forceinline__ void split_finish(const TcKernelParams& p, float& amax, const TileJob& j, bool ok, int et,
                                             int row, bool row_ok, int64_t base_c, int64_t base_d,
                                             volatile int* last_flag)
{
    __threadfence();
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (et == 0) {
        int last = 0;
        if (ok) last = (atomicAdd(p.counters + j.slot, 1) == j.nsplit - 1) ? 1 : 0;
        *last_flag = last;
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    const int is_last = *last_flag;
    if (is_last && ok) {
        __threadfence();
        const int chunks = p.bm / 32;
        for (int c = 0; c < chunks; ++c) {
            float v[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = 0.f;
            const size_t slab_elems = static_cast<size_t>(kTcTileN) * p.bm;
            const float* src0 = p.ws + static_cast<size_t>(j.slot) * p.tail_split * slab_elems +
                                static_cast<size_t>(c) * 32 * kTcTileN + row;
            for (int s = 0; s < j.nsplit; s += 2) {       // two slabs' loads in flight per step
                float a[32], b[32];
                const float* sa = src0 + static_cast<size_t>(s) * slab_elems;
                const bool two = s + 1 < j.nsplit;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    a[i] = __ldcg(sa + i * kTcTileN);
                    b[i] = two ? __ldcg(sa + slab_elems + i * kTcTileN) : 0.f;
                }
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] += a[i];
                if (two) {
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[i] += b[i];
                }
            }
            const int m = j.m0 + c * 32;
            if (row_ok && m < j.M) store_chunk<TD, EPI>(p, amax, j, base_c, base_d, m, v, p.out_trunc);
        }
        if (et == 0) p.counters[j.slot] = 0;   // ready for the next launch
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");   // last_flag is reused by the next tile
}

// C for one 32-output chunk, loaded ahead of its use (the epilogue keeps the next chunk's loads in
// flight while it finishes the current one).  16-bit outputs occupy cw[0..15] as packed pairs.
template <typename TD>
__device__ __forceinline__ void load_c_chunk(const TileJob& j, int64_t base_c, int m, uint32_t (&cw)[32])
{
    if constexpr (sizeof(TD) == 1) return;        // fp8 outputs take beta == 0: no C
    if (!(j.beta != 0.0f && j.C != nullptr) || m >= j.M) return;
    const char* cptr = static_cast<const char*>(j.C) + (base_c + m) * Out<TD>::kBytes;
    if (!j.out_t && m + 32 <= j.M && (reinterpret_cast<uintptr_t>(cptr) & 15) == 0) {
        constexpr int nvec = sizeof(TD) == 4 ? 8 : 4;
#pragma unroll
        for (int q = 0; q < nvec; ++q) {
            const uint4 w = __ldg(reinterpret_cast<const uint4*>(cptr) + q);
            cw[4 * q] = w.x;
            cw[4 * q + 1] = w.y;
            cw[4 * q + 2] = w.z;
            cw[4 * q + 3] = w.w;
        }
    } else {
#pragma unroll
        const int64_t cstep = j.out_t ? j.ldc : 1;
        for (int i = 0; i < 32; ++i) {
            const float c = (m + i < j.M) ? Out<TD>::load(j.C, base_c + (m + i) * cstep) : 0.f;
            if constexpr (sizeof(TD) == 4) {
                cw[i] = __float_as_uint(c);
            } else {
                // repack as the vector path does: element i in the low (even) / high (odd) half
                const uint32_t bits = (sizeof(TD) == 2 && std::is_same<TD, __half>::value)
                                          ? static_cast<uint32_t>(__half_as_ushort(__float2half_rn(c)))
                                          : (__float_as_uint(c) >> 16);
                if (i & 1) cw[i >> 1] |= bits << 16;
                else cw[i >> 1] = bits;
            }
        }
    }
}

// alpha*acc + beta*C for 32 outputs (C in registers from load_c_chunk), converted and packed into
// the output's bytes: 32 words for fp32, 16 for 16-bit types.
template <typename TD, bool EPI>
__device__ __forceinline__ void finish_pack(const TcKernelParams& p, float& amax, const TileJob& j, int m, bool row_ok,
                                            const uint32_t (&r)[32], const uint32_t (&cw)[32], int trunc, uint32_t* out)
{
    // rows past N and columns past M are computed but never stored: they stay out of the amax
    const bool use_c = (j.beta != 0.0f) && (j.C != nullptr);
    if constexpr (sizeof(TD) == 4) {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            const float a = __uint_as_float(r[i]);
            float o = use_c ? fmaf(j.alpha, a, j.beta * __uint_as_float(cw[i])) : j.alpha * a;
            if constexpr (EPI) o = epi_fn(p, m + i, row_ok && m + i < j.M, o, amax);
            out[i] = __float_as_uint(o);
        }
    } else if constexpr (sizeof(TD) == 1) {
        // E4M3: 32 outputs in 8 words (no C: fp8 outputs take beta == 0)
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            float o[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                o[t] = j.alpha * __uint_as_float(r[4 * q + t]);
                if constexpr (EPI) o[t] = epi_fn(p, m + 4 * q + t, row_ok && m + 4 * q + t < j.M, o[t], amax);
                o[t] = out_scale<TD>(p, o[t]);
            }
            out[q] = pack4_e4m3(o[0], o[1], o[2], o[3]);
        }
    } else {
        constexpr int is_half = std::is_same<TD, __half>::value ? 1 : 0;
#pragma unroll
        for (int h = 0; h < 16; ++h) {
            float c0 = 0.f, c1 = 0.f;
            if (use_c) unpack2(cw[h], is_half, c0, c1);
            const float a0 = __uint_as_float(r[2 * h]), a1 = __uint_as_float(r[2 * h + 1]);
            float o0 = use_c ? fmaf(j.alpha, a0, j.beta * c0) : j.alpha * a0;
            float o1 = use_c ? fmaf(j.alpha, a1, j.beta * c1) : j.alpha * a1;
            if constexpr (EPI) {
                o0 = epi_fn(p, m + 2 * h, row_ok && m + 2 * h < j.M, o0, amax);
                o1 = epi_fn(p, m + 2 * h + 1, row_ok && m + 2 * h + 1 < j.M, o1, amax);
            }
            out[h] = pack2(o0, o1, is_half, trunc);
        }
    }
}

// Finish a chunk with C already in registers (from load_c_chunk): v = alpha*acc + beta*C, store.
template <typename TD, bool EPI>
__device__ __forceinline__ void store_chunk_pre(const TcKernelParams& p, float& amax, const TileJob& j,
                                                int64_t base_d, int m, float (&acc)[32], const uint32_t (&cw)[32],
                                                int trunc)
{
    const bool use_c = (j.beta != 0.0f) && (j.C != nullptr);
    float c[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
        if constexpr (sizeof(TD) == 4) {
            c[i] = __uint_as_float(cw[i]);
        } else {
            const uint32_t w = cw[i >> 1];
            float lo, hi;
            unpack2(w, std::is_same<TD, __half>::value ? 1 : 0, lo, hi);
            c[i] = (i & 1) ? hi : lo;
        }
    }
    float o[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) o[i] = use_c ? fmaf(j.alpha, acc[i], j.beta * c[i]) : j.alpha * acc[i];
    if constexpr (EPI) {
#pragma unroll
        for (int i = 0; i < 32; ++i) o[i] = epi_fn(p, m + i, m + i < j.M, o[i], amax);
    }
    char* dptr = static_cast<char*>(j.D) + (base_d + m) * Out<TD>::kBytes;
    if (!j.out_t && m + 32 <= j.M && (reinterpret_cast<uintptr_t>(dptr) & 15) == 0) {
        if constexpr (sizeof(TD) == 4) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
                reinterpret_cast<float4*>(dptr)[q] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
        } else {
            constexpr int is_half = std::is_same<TD, __half>::value ? 1 : 0;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                reinterpret_cast<uint4*>(dptr)[q] =
                    make_uint4(pack2(o[8 * q], o[8 * q + 1], is_half, trunc), pack2(o[8 * q + 2], o[8 * q + 3], is_half, trunc),
                               pack2(o[8 * q + 4], o[8 * q + 5], is_half, trunc),
                               pack2(o[8 * q + 6], o[8 * q + 7], is_half, trunc));
        }
    } else {
        const int64_t dstep = j.out_t ? j.ldd : 1;
#pragma unroll
        for (int i = 0; i < 32; ++i)
            if (m + i < j.M) Out<TD>::store(j.D, base_d + (m + i) * dstep, o[i], trunc);
    }
}

// Hand a drained TMEM buffer back to the MMA issuer: one arrival per epilogue warp, on the leader
// CTA's barrier (a remote arrival when this CTA is the peer of a pair).
template <int CG>
__device__ __forceinline__ void release_tmem(uint64_t* bar, int lane)
{
    ptx::tc_fence_before();
    __syncwarp();
    if (lane == 0) {
        // the accumulator belongs to the pair's leader (the even rank of the pair)
        if constexpr (CG == 2) ptx::mbar_arrive_cluster(ptx::mapa_shared(ptx::smem_u32(bar), ptx::cluster_ctarank() & ~1u));
        else ptx::mbar_arrive(bar);
    }
}

// Split-k completion that keeps this split's own partial in TMEM: the partial was parked in the
// workspace for the other splits; if this CTA is the last of the tile to arrive it sums the
// partials in split order -- its own read back from TMEM, the others from the workspace with all of
// a chunk's loads in flight -- and runs the epilogue.  The TMEM buffer is released afterwards.
template <typename TD, int CG, bool EPI>
__device__ __forceinline__ void split_finish_tmem(const TcKernelParams& p, float& amax, const TileJob& j, bool ok,
                                                  int et, int lane,
                                                  int row, bool row_ok, int64_t base_c, int64_t base_d,
                                                  volatile int* last_flag, uint32_t tbase, uint64_t* tempty_bar)
{
    __threadfence();
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (et == 0) {
        int last = 0;
        if (ok) last = (atomicAdd(p.counters + j.slot, 1) == j.nsplit - 1) ? 1 : 0;
        *last_flag = last;
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    const int is_last = *last_flag;
    if (is_last && ok) {
        __threadfence();
        // CPS 32-column chunks per step (two for 16-bit outputs, one for fp32, whose C takes twice
        // the registers): their C values and every other split's partials are in flight together
        // (the reduction is latency-bound), summed in split order
        constexpr int CPS = sizeof(TD) == 2 ? 2 : 1;
        const int chunks = p.bm / 32;     // even: bm is 64, 128, 192 or 256
        const size_t slab_elems = static_cast<size_t>(kTcTileN) * p.bm;
        const float* base = p.ws + static_cast<size_t>(j.slot) * p.tail_split * slab_elems + row;
        for (int c = 0; c < chunks; c += CPS) {
            const int m0 = j.m0 + c * 32;
            uint32_t cw[CPS][32];
            if (CPS > 1 && row_ok) {
#pragma unroll
                for (int q = 0; q < CPS; ++q) load_c_chunk<TD>(j, base_c, m0 + 32 * q, cw[q]);
            }
            float v[CPS * 32];
#pragma unroll
            for (int i = 0; i < CPS * 32; ++i) v[i] = 0.f;
            for (int s = 0; s < j.nsplit; ++s) {
                if (s == j.split) {
#pragma unroll
                    for (int q = 0; q < CPS; ++q) {
                        uint32_t r[32];
                        __syncwarp();
                        ptx::tmem_ld32(tbase + (c + q) * 32, r);
#pragma unroll
                        for (int i = 0; i < 32; ++i) v[32 * q + i] += __uint_as_float(r[i]);
                    }
                } else {
                    float a[CPS * 32];
                    const float* src = base + static_cast<size_t>(s) * slab_elems + static_cast<size_t>(c) * 32 * kTcTileN;
#pragma unroll
                    for (int i = 0; i < CPS * 32; ++i) a[i] = __ldcg(src + i * kTcTileN);
#pragma unroll
                    for (int i = 0; i < CPS * 32; ++i) v[i] += a[i];
                }
            }
#pragma unroll
            for (int q = 0; q < CPS; ++q) {
                if (row_ok && m0 + 32 * q < j.M) {
                    float o[32];
#pragma unroll
                    for (int i = 0; i < 32; ++i) o[i] = v[32 * q + i];
                    if constexpr (CPS > 1) store_chunk_pre<TD, EPI>(p, amax, j, base_d, m0 + 32 * q, o, cw[q], p.out_trunc);
                    else store_chunk<TD, EPI>(p, amax, j, base_c, base_d, m0 + 32 * q, o, p.out_trunc);
                }
            }
        }
        if (et == 0) p.counters[j.slot] = 0;   // ready for the next launch
    }
    if (ok) release_tmem<CG>(tempty_bar, lane);
    asm volatile("bar.sync 1, 128;" ::: "memory");   // last_flag is reused by the next tile
}

// Bounded wait until *ctr >= target (acquire at GPU scope); false once limit_ns has passed.
__device__ __forceinline__ bool wait_counter_ge(const int* ctr, int target, uint64_t limit_ns)
{
    const uint64_t t0 = ptx::globaltimer();
    while (true) {
        int v;
        asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
        if (v >= target) return true;
        if (ptx::globaltimer() - t0 > limit_ns) return false;
        __nanosleep(64);
    }
}

// Split-k completion when every split unit of the launch is resident at once (all of them in the
// first round of the persistent schedule): each split has parked its partial tile, waits until the
// tile's other splits have too, then reduces its share of the tile -- 32-column chunks split,
// split + nsplit, ... -- summing the partials in split order (the same sums, bit for bit, as the
// last-arriver path) and runs their epilogue.  The tile counter counts arrivals up to nsplit, then
// finished shares up to 2 * nsplit, when the last one resets it for the next launch.
template <typename TD, int CG, bool EPI>
__device__ __forceinline__ void split_finish_parallel(const TcKernelParams& p, float& amax, const TileJob& j, bool& ok,
                                                      int et,
                                                      int lane, int row, bool row_ok, int64_t base_c, int64_t base_d,
                                                      volatile int* last_flag, uint64_t* tempty_bar,
                                                      volatile int* abort_flag, bool c_staged, uint32_t c_row)
{
    if (ok) release_tmem<CG>(tempty_bar, lane);     // this split's partial is in the workspace
    __threadfence();
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (et == 0) {
        int go = 0;
        if (ok) {
            atomicAdd(p.counters + j.slot, 1);
            go = wait_counter_ge(p.counters + j.slot, j.nsplit, p.timeout_ns) ? 1 : 0;
            if (!go) record_error(p, abort_flag, 16);
        }
        *last_flag = go;
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    const int go = *last_flag;
    if (go) {
        __threadfence();
        const int chunks = p.bm / 32;
        const size_t slab_elems = static_cast<size_t>(kTcTileN) * p.bm;
        const float* base = p.ws + static_cast<size_t>(j.slot) * p.tail_split * slab_elems + row;
        for (int c = j.split; c < chunks; c += j.nsplit) {
            const int m = j.m0 + c * 32;
            const bool live = row_ok && m < j.M;
            // two splits' partials at a time are in flight together (the reduction is
            // latency-bound), summed in split order
            float v[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = 0.f;
            for (int s = 0; s < j.nsplit; s += 2) {
                float a[32], b[32];
                const float* sa = base + static_cast<size_t>(s) * slab_elems + static_cast<size_t>(c) * 32 * kTcTileN;
                const bool two = s + 1 < j.nsplit;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    a[i] = __ldcg(sa + i * kTcTileN);
                    b[i] = two ? __ldcg(sa + slab_elems + i * kTcTileN) : 0.f;
                }
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] += a[i];
                if (two) {
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[i] += b[i];
                }
            }
            if (live) {
                if (c == j.split && c_staged) {
                    // this chunk's C row was copied into shared memory while the tile accumulated
                    // (16-byte unit u at u ^ (lane & 7))
                    uint32_t cw[32];
                    ptx::cp_async_wait0();
                    constexpr int NU = 32 * static_cast<int>(sizeof(TD)) / 16;
#pragma unroll
                    for (int u = 0; u < NU; ++u) {
                        const uint4 w4 = ptx::ld_shared_v4(c_row + static_cast<uint32_t>((u ^ (lane & 7)) * 16));
                        cw[4 * u] = w4.x;
                        cw[4 * u + 1] = w4.y;
                        cw[4 * u + 2] = w4.z;
                        cw[4 * u + 3] = w4.w;
                    }
                    store_chunk_pre<TD, EPI>(p, amax, j, base_d, m, v, cw, p.out_trunc);
                } else {
                    store_chunk<TD, EPI>(p, amax, j, base_c, base_d, m, v, p.out_trunc);
                }
            }
        }
    } else {
        ok = false;
    }
    if (c_staged) ptx::cp_async_wait0();   // the staging buffer is free again (also on the error path)
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (et == 0 && go) {
        // counts this split out of the tile: the last one resets the counter for the next launch.
        // No fence: the counter only orders the splits' waits (same-address atomics), and the next
        // launch's use of the workspace is ordered by the kernel boundary.
        if (atomicAdd(p.counters + j.slot, 1) == 2 * j.nsplit - 1) atomicExch(p.counters + j.slot, 0);
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");   // last_flag is reused by the next tile
}

template <int KIND, typename TD, int CL, bool EPI>
__global__ void __launch_bounds__(kTcThreads, 1) tc_gemm_kernel(const __grid_constant__ TcKernelParams p)
{
    // CL CTAs per cluster.  CL == 2: a CTA pair on two SMs works on one 256-row tile.  Each CTA
    // stages its own 128 rows of the n-side operand and its half of the m-side operand; the leader
    // (even rank) issues the pair MMAs, whose accumulator rows 0-127 live in the leader's TMEM and
    // 128-255 in the peer's.  The leader arms its full barriers with both CTAs' bytes and both CTAs'
    // TMA completions land on them; MMA completions are multicast to both CTAs, and both epilogues
    // release the leader's TMEM buffers with remote arrivals.
    // CL == 4: two such pairs on adjacent 256-row tiles with the same m range.  CTA r of one pair
    // needs the same m-side rows as CTA r of the other, so each loads half of them and multicasts
    // it to both (half the m-side L2 traffic); a ring slot is refilled only after both pairs' MMAs
    // have released it (each slot's empty barrier expects one commit from each pair's leader).
    constexpr int CG = CL >= 2 ? 2 : 1;         // CTAs per MMA (cta_group)
    constexpr int MC = CL / CG;                 // pairs sharing the m-side operand
    if (threadIdx.x == 0 && p.trace != nullptr) {
        trace_mark(p, TL_TRACE_ENTRY);
        trace_put(p, TL_TRACE_ENTRY_NS, global_ns());
        unsigned int smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        trace_put(p, TL_TRACE_SMID, smid);
    }
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t bmc = static_cast<uint32_t>(p.bm) / CG;            // m-side rows staged by this CTA
    const uint32_t tileN_bytes = kTcTileN * kTcRowBytes;
    const uint32_t stage_bytes = tileN_bytes + bmc * kTcRowBytes;
    // output staging for TMA stores: 4 epilogue warps x 32 rows x 128 bytes, 1024-byte aligned
    uint8_t* epi_stage = smem + static_cast<size_t>(p.stages) * stage_bytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(epi_stage + kTcEpiStageBytes);
    uint64_t* empty = full + kTcMaxStages;
    uint64_t* tfull = empty + kTcMaxStages;     // main accumulator buffers (per tile, or per chain)
    uint64_t* tempty = tfull + 2;
    uint64_t* sfull = tempty + 2;               // small-term accumulators (promotion with split terms)
    uint64_t* sempty = sfull + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sempty + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* last_flag = abort_flag + 1;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t rank = (CL > 1) ? ptx::cluster_ctarank() : 0u;
    const uint32_t pair_rank = rank & 1u;       // position within the CTA pair
    const uint32_t pair_base = rank & ~1u;      // the pair's leader
    const bool leader = (pair_rank == 0);
    const int64_t unit0 = (CL > 1) ? static_cast<int64_t>(ptx::cluster_id_x()) : static_cast<int64_t>(blockIdx.x);
    const int64_t units = (CL > 1) ? static_cast<int64_t>(ptx::ncluster_x()) : static_cast<int64_t>(gridDim.x);
    const bool promo = p.promote_kb > 0;
    const bool sep_small = promo && p.nterms > 1;
    // TMEM columns: main accumulator x2 (+ small-term accumulator x2 when they are kept apart)
    const uint32_t need_cols = static_cast<uint32_t>(p.bm) * (sep_small ? 4u : 2u);
    const uint32_t tmem_cols = need_cols <= 128 ? 128u : (need_cols <= 256 ? 256u : 512u);
    const uint32_t epi_arrivals = 4u * CG;     // one per epilogue warp of each CTA

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; ++s) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], MC);
        }
        for (int a = 0; a < 2; ++a) {
            ptx::mbar_init(&tfull[a], 1);
            ptx::mbar_init(&tempty[a], epi_arrivals);
            ptx::mbar_init(&sfull[a], 1);
            ptx::mbar_init(&sempty[a], epi_arrivals);
        }
        *abort_flag = 0;
        *last_flag = 0;
        ptx::fence_mbar_init();
        ptx::fence_proxy_async_smem();
    }
    if (warp == 1) {
        if constexpr (CG == 2) {
            ptx::tmem_alloc_pair(tmem_slot, tmem_cols);
            ptx::tmem_relinquish_pair();
        } else {
            ptx::tmem_alloc(tmem_slot, tmem_cols);
            ptx::tmem_relinquish();
        }
    }
    if (warp == 0 && lane == 0 && p.group == nullptr) {
        for (int v = 0; v < p.nterms; ++v) {
            ptx::prefetch_tmap(&p.tmN[p.term_n[v]]);
            ptx::prefetch_tmap(&p.tmM[p.term_m[v]]);
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    if constexpr (CL > 1) ptx::cluster_sync();     // peer barriers initialised before any remote arrive
    ptx::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    if (threadIdx.x == 0) trace_mark(p, TL_TRACE_SETUP);
    // Launched as a programmatic dependent: everything above (barrier set-up, TMEM allocation,
    // descriptor prefetch) may have run while the previous kernel in the stream was finishing.
    // Wait for that grid to complete (its writes visible) before touching global memory, then let
    // the next dependent grid start its own set-up as soon as SMs free up.
    ptx::grid_dep_wait();
    ptx::grid_dep_launch_dependents();
    if (threadIdx.x == 0) trace_mark(p, TL_TRACE_DEP);
    const int nvirt = p.nterms;
    const uint64_t tlim = p.timeout_ns;

    if (warp == 0) {
        // ------------------------------------------------------------------ TMA producer (each CTA)
        // One flat loop over (k-block, product) per tile, run by the whole warp in step: its waits
        // (single PTX blocks, voted across the warp) and bookkeeping are warp-uniform, and one
        // elected lane issues the copies.
        {
            uint32_t stage = 0, phase = 0;
            constexpr int W = kTcRowBytes / (KIND == 0 ? 2 : 1);   // elements per 128-byte row
            const int n_mn = p.n_mn_major, m_mn = p.m_mn_major;
            const int nstages = p.stages;
            bool ok = true;
            int4 u_next = load_unit(p, unit0);
            for (int64_t w = unit0; w < p.total_work && ok; w += units) {
                const int4 u = u_next;
                u_next = load_unit(p, w + units);      // in flight during this tile
                TileJob j;
                get_job(p, w, u, j);
                const int n0 = j.n0 + static_cast<int>(rank) * kTcTileN;
                const int m0 = j.m0 + static_cast<int>(pair_rank * bmc);
                const int total = (j.kb1 - j.kb0) * nvirt;
                int kb = j.kb0, v = 0;
                // timeline stamps stay outside the k-block loops (a branch there slows the issue)
                if (w == unit0 && lane == 0) trace_mark(p, TL_TRACE_LOAD_FIRST);
                for (int i = 0; i < total; ++i) {
                    if (!__all_sync(0xffffffffu, ptx::mbar_wait(&empty[stage], phase ^ 1u, tlim))) {
                        if (lane == 0) record_error(p, abort_flag, 1);
                        ok = false;
                        break;
                    }
                    // the timeout-path test issues nothing: the full barriers never complete, the
                    // MMA and epilogue waits run out, and no copy is left in flight
                    if (!p.debug_skip_loads && ptx::elect_one()) {
                        uint8_t* sN = smem + static_cast<size_t>(stage) * stage_bytes;
                        uint8_t* sM = sN + tileN_bytes;
                        // split-precision products, smallest first (term table set by the host)
                        const void* mapN = p.group ? j.tmN : static_cast<const void*>(&p.tmN[p.term_n[v]]);
                        const void* mapM = p.group ? j.tmM : static_cast<const void*>(&p.tmM[p.term_m[v]]);
                        const int k0 = kb * W;
                        if constexpr (CG == 2) {
                            // the leader arms its full barrier with both CTAs' bytes; the peer's loads
                            // only complete transactions on it (they cannot run a phase ahead: the
                            // peer refills a slot only after the leader's MMAs released it)
                            const uint32_t fb = ptx::mapa_shared(ptx::smem_u32(&full[stage]), pair_base);
                            if (leader) ptx::mbar_arrive_expect_tx(&full[stage], 2u * stage_bytes);
                            if (!n_mn) {
                                ptx::tma_load_3d_pair(sN, mapN, fb, k0, n0, j.b);
                            } else {
#pragma unroll
                                for (int c = 0; c < kTcTileN / W; ++c)
                                    ptx::tma_load_3d_pair(sN + c * W * kTcRowBytes, mapN, fb, n0 + c * W, k0, j.b);
                            }
                            if constexpr (MC == 2) {
                                // this CTA's half of the m rows shared with CTA pair_rank of the other
                                // pair; the copy lands in both and is counted on each pair's leader
                                const int half = static_cast<int>(rank >> 1);
                                const uint16_t mask = static_cast<uint16_t>((1u << pair_rank) | (1u << (pair_rank + 2)));
                                if (!m_mn)
                                    ptx::tma_load_3d_pair_mc(sM + half * (bmc / 2) * kTcRowBytes, mapM, fb, mask, k0,
                                                             m0 + half * static_cast<int>(bmc / 2), j.b);
                                else
                                    ptx::tma_load_3d_pair_mc(sM + half * W * kTcRowBytes, mapM, fb, mask,
                                                             m0 + half * W, k0, j.b);
                            } else if (!m_mn) {
                                ptx::tma_load_3d_pair(sM, mapM, fb, k0, m0, j.b);
                            } else {
#pragma unroll
                                for (int c = 0; c < 4; ++c)      // bmc / W <= 4 chunks
                                    if (c * W < static_cast<int>(bmc))
                                        ptx::tma_load_3d_pair(sM + c * W * kTcRowBytes, mapM, fb, m0 + c * W, k0, j.b);
                            }
                        } else {
                            ptx::mbar_arrive_expect_tx(&full[stage], stage_bytes);
                            if (!n_mn) {
                                ptx::tma_load_3d(sN, mapN, &full[stage], k0, n0, j.b);
                            } else {
#pragma unroll
                                for (int c = 0; c < kTcTileN / W; ++c)
                                    ptx::tma_load_3d(sN + c * W * kTcRowBytes, mapN, &full[stage], n0 + c * W, k0, j.b);
                            }
                            if (!m_mn) {
                                ptx::tma_load_3d(sM, mapM, &full[stage], k0, m0, j.b);
                            } else {
#pragma unroll
                                for (int c = 0; c < 4; ++c)      // bmc / W <= 4 chunks
                                    if (c * W < static_cast<int>(bmc))
                                        ptx::tma_load_3d(sM + c * W * kTcRowBytes, mapM, &full[stage], m0 + c * W, k0, j.b);
                            }
                        }
                    }
                    __syncwarp();
                    if (++stage == static_cast<uint32_t>(nstages)) {
                        stage = 0;
                        phase ^= 1u;
                    }
                    if (++v == nvirt) {
                        v = 0;
                        ++kb;
                    }
                }
                if (w == unit0 && lane == 0) trace_mark(p, TL_TRACE_LOAD_LAST);
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------------ MMA issuer (leader CTA)
        // Without promotion a tile's whole k range accumulates in one TMEM buffer (two buffers
        // alternate between tiles).  With promotion the A0*B0 product restarts its accumulation
        // every promote_kb k-blocks in the alternate buffer (the epilogue drains each chain into
        // fp32 registers), and the small split-precision products accumulate for the whole tile in
        // a separate pair of buffers.  One flat loop per tile over (k-block, product), run by the
        // whole warp in step (uniform waits and bookkeeping); one elected lane issues the MMAs and
        // their commits.
        if (leader) {
            uint32_t stage = 0, phase = 0, mbuf = 0, mph = 0, sbuf = 0, sph = 0;
            const uint16_t pair_mask = static_cast<uint16_t>(0x3u << pair_base);
            const uint32_t idesc = p.idesc;
            const uint32_t n_kstep = p.n_kstep, m_kstep = p.m_kstep, n_lbo = p.n_lbo, m_lbo = p.m_lbo;
            const uint32_t bmu = static_cast<uint32_t>(p.bm);
            const int nstages = p.stages;
            bool ok = true;
            int4 u_next = load_unit(p, unit0);
            for (int64_t w = unit0; w < p.total_work && ok; w += units) {
                const int4 u = u_next;
                u_next = load_unit(p, w + units);      // in flight during this tile
                TileJob j;
                get_job(p, w, u, j);
                const int nkb = j.kb1 - j.kb0;
                if (nkb <= 0) continue;                 // an empty unit of a balanced split
                const int chunk = promo ? p.promote_kb : nkb;
                if (sep_small) {
                    if (!__all_sync(0xffffffffu, ptx::mbar_wait(&sempty[sbuf], sph ^ 1u, tlim))) {
                        if (lane == 0) record_error(p, abort_flag, 2);
                        break;
                    }
                    ptx::tc_fence_after();
                }
                if (nkb > 0) {
                    if (!__all_sync(0xffffffffu, ptx::mbar_wait(&tempty[mbuf], mph ^ 1u, tlim))) {
                        if (lane == 0) record_error(p, abort_flag, 2);
                        break;
                    }
                    ptx::tc_fence_after();
                }
                bool main_started = false, small_started = false;
                const int total = nkb * nvirt;
                int v = 0, kb_in_chain = 0;
                if (p.trace != nullptr && w == unit0 && total > 0) {
                    // timeline: the first stage's arrival, waited for here (the loop's own wait on
                    // it then passes at once) so that the k-block loop carries no stamp
                    ptx::mbar_wait(&full[stage], phase, tlim);
                    if (lane == 0) trace_mark(p, TL_TRACE_MMA_FIRST);
                    __syncwarp();
                }
                for (int i = 0; i < total; ++i) {
                    if (!__all_sync(0xffffffffu, ptx::mbar_wait(&full[stage], phase, tlim))) {
                        if (lane == 0) record_error(p, abort_flag, 4);
                        ok = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const bool is_main = !sep_small || v == nvirt - 1;
                    const uint32_t d_tmem = tmem_base + (is_main ? mbuf * bmu : (2u + sbuf) * bmu);
                    const bool started = is_main ? main_started : small_started;
                    const uint32_t sN = ptx::smem_u32(smem + static_cast<size_t>(stage) * stage_bytes);
                    const uint32_t sM = sN + tileN_bytes;
                    if (ptx::elect_one()) {
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks) {
                            const uint64_t adesc = ptx::sdesc_sw128(sN + ks * n_kstep, n_lbo, 1024);
                            const uint64_t bdesc = ptx::sdesc_sw128(sM + ks * m_kstep, m_lbo, 1024);
                            const uint32_t accumulate = (started || ks > 0) ? 1u : 0u;
                            if constexpr (CG == 2) {
                                if (KIND == 0) ptx::mma_f16_pair(d_tmem, adesc, bdesc, idesc, accumulate);
                                else ptx::mma_f8_pair(d_tmem, adesc, bdesc, idesc, accumulate);
                            } else {
                                if (KIND == 0) ptx::mma_f16(d_tmem, adesc, bdesc, idesc, accumulate);
                                else ptx::mma_f8(d_tmem, adesc, bdesc, idesc, accumulate);
                            }
                        }
                        // both pairs' ring slots are released (MC == 2: every CTA of the cluster)
                        if constexpr (CG == 2) ptx::mma_commit_pair(&empty[stage], MC == 2 ? 0xF : 0x3);
                        else ptx::mma_commit(&empty[stage]);
                    }
                    __syncwarp();
                    main_started = main_started || is_main;
                    small_started = small_started || !is_main;
                    if (++stage == static_cast<uint32_t>(nstages)) {
                        stage = 0;
                        phase ^= 1u;
                    }
                    if (++v == nvirt) {
                        v = 0;
                        // end of a chain of the main product: hand it to the epilogue, continue in
                        // the other buffer (a tile's last chain is handed over after the loop)
                        if (++kb_in_chain == chunk && i + 1 < total) {
                            if (ptx::elect_one()) {
                                if constexpr (CG == 2) ptx::mma_commit_pair(&tfull[mbuf], pair_mask);
                                else ptx::mma_commit(&tfull[mbuf]);
                            }
                            __syncwarp();
                            mbuf ^= 1u;
                            if (mbuf == 0) mph ^= 1u;
                            kb_in_chain = 0;
                            main_started = false;
                            if (!__all_sync(0xffffffffu, ptx::mbar_wait(&tempty[mbuf], mph ^ 1u, tlim))) {
                                if (lane == 0) record_error(p, abort_flag, 2);
                                ok = false;
                                break;
                            }
                            ptx::tc_fence_after();
                        }
                    }
                }
                if (!ok) break;
                if (ptx::elect_one()) {
                    if (nkb > 0) {
                        if constexpr (CG == 2) ptx::mma_commit_pair(&tfull[mbuf], pair_mask);
                        else ptx::mma_commit(&tfull[mbuf]);
                    }
                    if (sep_small) {
                        if constexpr (CG == 2) ptx::mma_commit_pair(&sfull[sbuf], pair_mask);
                        else ptx::mma_commit(&sfull[sbuf]);
                    }
                }
                __syncwarp();
                if (w == unit0 && lane == 0) trace_mark(p, TL_TRACE_MMA_LAST);
                if (nkb > 0) {
                    mbuf ^= 1u;
                    if (mbuf == 0) mph ^= 1u;
                }
                if (sep_small) {
                    sbuf ^= 1u;
                    if (sbuf == 0) sph ^= 1u;
                }
            }
        }
    } else {
        // ------------------------------------------------------------------ epilogue (4 warps, each CTA)
        // All four warps run the same loop and, in split-k mode, the same named barriers: after a
        // timed-out wait a warp keeps the control flow and only skips the work, so no warp can be
        // left waiting at bar.sync 1 for one that gave up.
        const int quarter = warp & 3;             // TMEM lanes 32*quarter .. +31
        const int row = quarter * 32 + lane;      // tile row = problem n offset within this CTA
        const int et = threadIdx.x - 64;          // 0..127
        const uint32_t lane_off = static_cast<uint32_t>(quarter * 32) << 16;
        uint32_t mbuf = 0, mph = 0, sbuf = 0, sph = 0;
        const int chunks = p.bm / 32;
        bool ok = true;
        float amax = 0.0f;                        // fused epilogue: this thread's max |output|
        unsigned long long units_done = 0;
        for (int64_t w = unit0; w < p.total_work; w += units) {
            const int4 u = load_unit(p, w);      // the epilogue trails the MMAs: no need to load ahead
            TileJob j;
            get_job(p, w, u, j);
            if (j.kb1 <= j.kb0) continue;             // an empty unit of a balanced split
            ++units_done;
            const bool tr = (et == 0 && w == unit0);  // timeline stamps: the first tile, one thread
            j.n0 += static_cast<int>(rank) * kTcTileN;
            j.slot = j.slot * CL + rank;              // split-k slabs and counters per CTA
            const int n = j.n0 + row;
            const bool row_ok = n < j.N;
            // this thread's row n of the output: a contiguous run of m, or with a transposed output
            // one element of each of the columns m (stride ld)
            const int64_t base_d = static_cast<int64_t>(j.b) * p.stride_d + static_cast<int64_t>(n) * (j.out_t ? 1 : j.ldd);
            const int64_t base_c = static_cast<int64_t>(j.b) * p.stride_c + static_cast<int64_t>(n) * (j.out_t ? 1 : j.ldc);
            if (ok && row_ok && !j.out_t && j.beta != 0.0f && j.C != nullptr && (j.nsplit == 1 || j.split == j.nsplit - 1)) {
                // C does not depend on the accumulator: start pulling this row's segment into L2
                // while the tile is still accumulating
                const char* cp = static_cast<const char*>(j.C) + (base_c + j.m0) * static_cast<int64_t>(sizeof(TD));
                const int cbytes = (min(p.bm, j.M - j.m0)) * static_cast<int>(sizeof(TD));
                for (int off = 0; off < cbytes; off += 128)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(cp + off));
            }
            if (ok && j.out_t && j.beta != 0.0f && j.C != nullptr) {
                // transposed output: the warp's C is a 64- or 128-byte run of each column; lane L
                // pulls column L of every 32-column chunk into L2 (both lines a run may touch)
                const int nrow0 = j.n0 + quarter * 32;
                if (nrow0 < j.N) {
                    for (int c = 0; c < chunks; ++c) {
                        const int ccol = j.m0 + c * 32 + lane;
                        if (ccol >= j.M) break;
                        const char* cp = static_cast<const char*>(j.C) +
                                         (static_cast<int64_t>(j.b) * p.stride_c + static_cast<int64_t>(ccol) * j.ldc + nrow0) *
                                             static_cast<int64_t>(sizeof(TD));
                        const int last = (min(32, j.N - nrow0) * static_cast<int>(sizeof(TD))) - 1;
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(cp));
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(cp + last));
                    }
                }
            }
            if (promo) {
                // ---- promotion: sum the A0*B0 chains (and the small terms) in fp32 registers; bm == 128
                float run[128];
#pragma unroll
                for (int i = 0; i < 128; ++i) run[i] = 0.f;
                const int nkb = j.kb1 - j.kb0;
                const int nchain = (nkb + p.promote_kb - 1) / p.promote_kb;
                for (int c = 0; c < nchain; ++c) {
                    bool got = ok && ptx::mbar_wait(&tfull[mbuf], mph, tlim, abort_flag);
                    got = __all_sync(0xffffffffu, got);
                    if (ok && !got) {
                        if (lane == 0) record_error(p, abort_flag, 8);
                        ok = false;
                    }
                    if (ok) {
                        ptx::tc_fence_after();
                        const uint32_t tb = tmem_base + lane_off + mbuf * static_cast<uint32_t>(p.bm);
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            uint32_t r[32];
                            __syncwarp();
                            ptx::tmem_ld32(tb + q * 32, r);
#pragma unroll
                            for (int i = 0; i < 32; ++i) run[q * 32 + i] += __uint_as_float(r[i]);
                        }
                        release_tmem<CG>(&tempty[mbuf], lane);
                    }
                    mbuf ^= 1u;
                    if (mbuf == 0) mph ^= 1u;
                }
                if (sep_small) {
                    bool got = ok && ptx::mbar_wait(&sfull[sbuf], sph, tlim, abort_flag);
                    got = __all_sync(0xffffffffu, got);
                    if (ok && !got) {
                        if (lane == 0) record_error(p, abort_flag, 8);
                        ok = false;
                    }
                    if (ok) {
                        ptx::tc_fence_after();
                        const uint32_t tb = tmem_base + lane_off + (2u + sbuf) * static_cast<uint32_t>(p.bm);
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            uint32_t r[32];
                            __syncwarp();
                            ptx::tmem_ld32(tb + q * 32, r);
#pragma unroll
                            for (int i = 0; i < 32; ++i) run[q * 32 + i] += __uint_as_float(r[i]);
                        }
                        release_tmem<CG>(&sempty[sbuf], lane);
                    }
                    sbuf ^= 1u;
                    if (sbuf == 0) sph ^= 1u;
                }
                if (tr) trace_mark(p, TL_TRACE_ACC_READY);
                if (j.nsplit == 1) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int m = j.m0 + q * 32;
                        if (ok && row_ok && m < j.M) {
                            float v[32];
#pragma unroll
                            for (int i = 0; i < 32; ++i) v[i] = run[q * 32 + i];
                            store_chunk<TD, EPI>(p, amax, j, base_c, base_d, m, v, p.out_trunc);
                        }
                    }
                    if (tr) trace_mark(p, TL_TRACE_STORED);
                } else {
                    float* slab = p.ws + (static_cast<size_t>(j.slot) * p.tail_split + j.split) *
                                             (static_cast<size_t>(kTcTileN) * p.bm);
                    if (ok) {
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            float* dst = slab + static_cast<size_t>(q) * 32 * kTcTileN + row;
#pragma unroll
                            for (int i = 0; i < 32; ++i) __stcg(dst + i * kTcTileN, run[q * 32 + i]);
                        }
                    }
                    if (tr) trace_mark(p, TL_TRACE_STORED);
                    split_finish<TD, EPI>(p, amax, j, ok, et, row, row_ok, base_c, base_d, last_flag);
                    if (tr) trace_mark(p, TL_TRACE_REDUCED);
                }
                continue;
            }
            // ---- one TMEM accumulator per tile
            // parallel split-k: this split finishes 32-column chunk `split` of the tile.  Its C does
            // not depend on the accumulator: each thread copies its row of it into the warp's
            // output staging buffer (free in this mode: no TMA store is in flight from it) while the
            // tile accumulates.
            bool c_staged = false;
            const uint32_t c_row = ptx::smem_u32(epi_stage) + static_cast<uint32_t>(quarter) * 4096u +
                                   static_cast<uint32_t>(lane) * 128u;
            if constexpr (sizeof(TD) >= 2) {
                const int mc = j.m0 + j.split * 32;
                if (p.par_reduce && !j.out_t && j.nsplit > 1 && j.beta != 0.0f && j.C != nullptr && j.split * 32 < p.bm) {
                    if (lane == 0) ptx::bulk_wait_read0();
                    __syncwarp();
                    const char* cptr = static_cast<const char*>(j.C) + (base_c + mc) * static_cast<int64_t>(sizeof(TD));
                    if (row_ok && mc + 32 <= j.M && (reinterpret_cast<uintptr_t>(cptr) & 15) == 0) {
                        constexpr int NU = 32 * static_cast<int>(sizeof(TD)) / 16;
#pragma unroll
                        for (int u = 0; u < NU; ++u)
                            ptx::cp_async16(c_row + static_cast<uint32_t>((u ^ (lane & 7)) * 16), cptr + 16 * u);
                        c_staged = true;
                    }
                    ptx::cp_async_commit();
                }
            }
            bool got = ok && ptx::mbar_wait(&tfull[mbuf], mph, tlim, abort_flag);
            got = __all_sync(0xffffffffu, got);
            if (ok && !got) {
                if (lane == 0) record_error(p, abort_flag, 8);
                ok = false;
            }
            const uint32_t tbase = tmem_base + lane_off + mbuf * static_cast<uint32_t>(p.bm);
            if (ok) ptx::tc_fence_after();
            if (tr) trace_mark(p, TL_TRACE_ACC_READY);
            // A staged TMA store costs a round trip per 32 rows (the one 4 KB buffer per warp is
            // refilled only after the previous store has read it): hidden behind the next tile's
            // main loop, but exposed on a CTA's last tile, which uses the direct stores instead
            // when beta == 0 (with a C operand to read, the staged path measured faster).
            const bool direct = p.direct_last && !j.out_t && j.beta == 0.0f && w + units >= p.total_work;
            if constexpr (sizeof(TD) >= 2 && !EPI) {
                if (j.out_t && j.nsplit == 1 && j.tmD != nullptr) {
                    // transposed output: a warp's 32 rows are 32 consecutive elements of D's columns,
                    // so each 32-column chunk is one 32 x 32 box of D, staged [column][row] (two boxes
                    // per 4 KB buffer for 16-bit outputs, one for fp32) and written by one TMA store;
                    // a box's buffer is refilled once the store two (16-bit) or one (fp32) back has
                    // read it.  With beta, lane L first brings column L of the chunk's C (contiguous
                    // in memory) into the box, and every lane then replaces its row of C by D.
                    constexpr int CB = 32 * 32 * static_cast<int>(sizeof(TD));   // bytes per box
                    constexpr int NB = 4096 / CB;
                    constexpr int COLB = CB / 32;                                  // bytes per box column
                    const int nrow0 = j.n0 + quarter * 32;
                    const bool use_c = j.beta != 0.0f && j.C != nullptr;
                    for (int c = 0; c < chunks && ok; ++c) {
                        const int m = j.m0 + c * 32;
                        if (lane == 0) {
                            if constexpr (NB == 2) ptx::bulk_wait_read1();
                            else ptx::bulk_wait_read0();
                        }
                        __syncwarp();
                        uint8_t* box = epi_stage + quarter * 4096 + (c % NB) * CB;
                        const uint32_t ba = ptx::smem_u32(box);
                        if (use_c) {
                            const int ccol = m + lane;
                            if (ccol < j.M) {
                                const int64_t cbase = static_cast<int64_t>(j.b) * p.stride_c +
                                                      static_cast<int64_t>(ccol) * j.ldc + nrow0;
                                const char* src = static_cast<const char*>(j.C) + cbase * static_cast<int64_t>(sizeof(TD));
                                if (nrow0 + 32 <= j.N && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
                                    // every load of the column is in flight before the first store
                                    uint4 v4[COLB / 16];
#pragma unroll
                                    for (int q = 0; q < COLB / 16; ++q) v4[q] = __ldg(reinterpret_cast<const uint4*>(src) + q);
#pragma unroll
                                    for (int q = 0; q < COLB / 16; ++q)
                                        ptx::st_shared_v4(ba + static_cast<uint32_t>(lane * COLB + q * 16), v4[q].x, v4[q].y,
                                                          v4[q].z, v4[q].w);
                                } else {
#pragma unroll 1
                                    for (int rr = 0; rr < 32; ++rr) {
                                        const float cv = (nrow0 + rr < j.N) ? Out<TD>::load(j.C, cbase + rr) : 0.f;
                                        const uint32_t a = ba + static_cast<uint32_t>(lane * COLB + rr * static_cast<int>(sizeof(TD)));
                                        if constexpr (sizeof(TD) == 4) ptx::st_shared_u32(a, __float_as_uint(cv));
                                        else if constexpr (std::is_same<TD, __half>::value)
                                            ptx::st_shared_u16(a, __half_as_ushort(__float2half_rn(cv)));
                                        else ptx::st_shared_u16(a, static_cast<uint16_t>(__float_as_uint(cv) >> 16));
                                    }
                                }
                            }
                            __syncwarp();
                        }
                        uint32_t r[32];
                        __syncwarp();
                        ptx::tmem_ld32(tbase + c * 32, r);
                        if (c == chunks - 1) release_tmem<CG>(&tempty[mbuf], lane);
#pragma unroll
                        for (int i = 0; i < 32; ++i) {
                            const uint32_t a = ba + static_cast<uint32_t>((i * 32 + lane) * static_cast<int>(sizeof(TD)));
                            const float acc = __uint_as_float(r[i]);
                            if constexpr (sizeof(TD) == 4) {
                                const float o = use_c ? fmaf(j.alpha, acc, j.beta * __uint_as_float(ptx::ld_shared_u32(a)))
                                                      : j.alpha * acc;
                                ptx::st_shared_u32(a, __float_as_uint(o));
                            } else {
                                constexpr bool half = std::is_same<TD, __half>::value;
                                float cf = 0.f;
                                if (use_c) {
                                    const uint32_t bits = ptx::ld_shared_u16(a);
                                    cf = half ? __half2float(__ushort_as_half(static_cast<unsigned short>(bits)))
                                              : __uint_as_float(bits << 16);
                                }
                                const float o = use_c ? fmaf(j.alpha, acc, j.beta * cf) : j.alpha * acc;
                                uint16_t ob;
                                if constexpr (half) ob = __half_as_ushort(__float2half_rn(o));
                                else ob = p.out_trunc ? static_cast<uint16_t>(__float_as_uint(o) >> 16)
                                                      : __bfloat16_as_ushort(__float2bfloat16_rn(o));
                                ptx::st_shared_u16(a, ob);
                            }
                        }
                        ptx::fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0 && m < j.M && nrow0 < j.N) {
                            ptx::tma_store_3d(j.tmD, box, nrow0, m, j.b);
                            ptx::bulk_commit();
                        }
                    }
                    if (tr) trace_mark(p, TL_TRACE_STORED);
                    mbuf ^= 1u;
                    if (mbuf == 0) mph ^= 1u;
                    continue;
                }
            }
            if (j.nsplit == 1 && j.tmD != nullptr && !direct) {
                // each warp stages its 32 rows x 128 bytes of output (128-byte swizzle: 16-byte unit
                // u of row r sits at u ^ (r & 7)) and writes them with one TMA store; the tensor
                // map clips the ragged edges.  One staging buffer per warp: before refilling it the
                // issuing lane waits until the previous store has read it.
                constexpr int CPS = static_cast<int>(4 / sizeof(TD));    // 32-column chunks per 128 bytes
                const uint32_t stg = ptx::smem_u32(epi_stage) + static_cast<uint32_t>(quarter) * 4096u;
                const int nrow0 = j.n0 + quarter * 32;
                for (int c0 = 0; c0 < chunks && ok; c0 += CPS) {
                    const int m = j.m0 + c0 * 32;
                    if (lane == 0) ptx::bulk_wait_read0();
                    __syncwarp();
                    const uint32_t rowaddr = stg + static_cast<uint32_t>(lane) * 128u;
#pragma unroll
                    for (int q = 0; q < CPS; ++q) {
                        uint32_t cw[32];
                        if (row_ok) load_c_chunk<TD>(j, base_c, m + 32 * q, cw);
                        uint32_t r[32];
                        __syncwarp();
                        ptx::tmem_ld32(tbase + (c0 + q) * 32, r);
                        uint32_t w[32 / CPS];
                        finish_pack<TD, EPI>(p, amax, j, m + 32 * q, row_ok, r, cw, p.out_trunc, w);
#pragma unroll
                        for (int uu = 0; uu < 8 / CPS; ++uu) {
                            const int u = q * (8 / CPS) + uu;
                            ptx::st_shared_v4(rowaddr + static_cast<uint32_t>((u ^ (lane & 7)) * 16), w[4 * uu],
                                              w[4 * uu + 1], w[4 * uu + 2], w[4 * uu + 3]);
                        }
                    }
                    if (c0 + CPS >= chunks) release_tmem<CG>(&tempty[mbuf], lane);
                    ptx::fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0 && m < j.M && nrow0 < j.N) {
                        ptx::tma_store_3d(j.tmD, epi_stage + quarter * 4096, m, nrow0, j.b);
                        ptx::bulk_commit();
                    }
                }
                if (tr) trace_mark(p, TL_TRACE_STORED);
            } else if (j.nsplit == 1) {
                // output TMA cannot address (unaligned D): 16-byte vector stores per thread
                for (int c = 0; c < chunks && ok; ++c) {
                    const int m = j.m0 + c * 32;
                    uint32_t r[32];
                    __syncwarp();
                    ptx::tmem_ld32(tbase + c * 32, r);
                    if (c == chunks - 1) release_tmem<CG>(&tempty[mbuf], lane);
                    if (row_ok && m < j.M) {
                        float v[32];
#pragma unroll
                        for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
                        store_chunk<TD, EPI>(p, amax, j, base_c, base_d, m, v, p.out_trunc);
                    }
                }
                if (tr) trace_mark(p, TL_TRACE_STORED);
            } else {
                // split-k: park this split's partial tile, layout [chunk][column][row] (coalesced)
                float* slab = p.ws + (static_cast<size_t>(j.slot) * p.tail_split + j.split) *
                                         (static_cast<size_t>(kTcTileN) * p.bm);
                for (int c = 0; c < chunks && ok; ++c) {
                    uint32_t r[32];
                    __syncwarp();
                    ptx::tmem_ld32(tbase + c * 32, r);
                    float* dst = slab + static_cast<size_t>(c) * 32 * kTcTileN + row;
#pragma unroll
                    for (int i = 0; i < 32; ++i) __stcg(dst + i * kTcTileN, __uint_as_float(r[i]));
                }
                if (tr) trace_mark(p, TL_TRACE_STORED);
                if (p.par_reduce)
                    split_finish_parallel<TD, CG, EPI>(p, amax, j, ok, et, lane, row, row_ok, base_c, base_d, last_flag,
                                                  &tempty[mbuf], abort_flag, c_staged, c_row);
                else
                    split_finish_tmem<TD, CG, EPI>(p, amax, j, ok, et, lane, row, row_ok, base_c, base_d, last_flag, tbase,
                                              &tempty[mbuf]);
                if (tr) trace_mark(p, TL_TRACE_REDUCED);
            }
            mbuf ^= 1u;
            if (mbuf == 0) mph ^= 1u;
        }
        if (et == 0) {
            trace_mark(p, TL_TRACE_EPI_END);
            trace_put(p, TL_TRACE_TILES, units_done);
        }
        if constexpr (EPI) {
            if (p.epi_amax != nullptr) {
                // max |output| of the warp, then one atomic per warp (non-negative floats order as ints)
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, off));
                if (lane == 0) atomicMax(reinterpret_cast<int*>(p.epi_amax), __float_as_int(amax));
            }
        }
    }

    if (warp >= 2 && lane == 0) ptx::bulk_wait0();   // the epilogue's TMA stores have completed
    ptx::tc_fence_before();
    __syncthreads();
    if constexpr (CL > 1) ptx::cluster_sync();     // no remote arrival, multicast or pair MMA still targets us
    if (warp == 1) {
        ptx::tc_fence_after();
        if constexpr (CG == 2) ptx::tmem_dealloc_pair(tmem_base, tmem_cols);
        else ptx::tmem_dealloc(tmem_base, tmem_cols);
        if (lane == 0 && p.trace != nullptr) {
            trace_mark(p, TL_TRACE_EXIT);
            trace_put(p, TL_TRACE_EXIT_NS, global_ns());
        }
    }
}

// ---- host side ------------------------------------------------------------------------------------
// ---- launch (templates; instantiated in the generated instance units) ---------------------------
bool pdl_enabled();

template <int KIND, typename TD, int CL, bool EPI = false>
tl_status launch_kernel(const TcKernelParams& kp, int grid, size_t smem, cudaStream_t stream)
{
    auto kern = tc_gemm_kernel<KIND, TD, CL, EPI>;
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [&] {
        attr_err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    });
    if (attr_err != cudaSuccess) return cuda_fail(attr_err, "cudaFuncSetAttribute(tc_gemm_kernel)");
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(static_cast<unsigned>(grid), 1, 1);
    cfg.blockDim = dim3(kTcThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[2];
    int na = 0;
    if (pdl_enabled()) {
        // programmatic dependent launch: this grid's prologue may overlap the previous kernel's tail
        // (the kernel waits for the previous grid before its first global-memory access)
        attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    if constexpr (CL > 1) {
        attr[na].id = cudaLaunchAttributeClusterDimension;
        attr[na].val.clusterDim.x = CL;
        attr[na].val.clusterDim.y = 1;
        attr[na].val.clusterDim.z = 1;
        ++na;
    }
    cfg.attrs = attr;
    cfg.numAttrs = na;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, kp);
    if (e != cudaSuccess) return cuda_fail(e, CL > 1 ? "cudaLaunchKernelEx(tc_gemm_kernel, cluster launch)"
                                                     : "cudaLaunchKernelEx(tc_gemm_kernel)");
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "tc_gemm_kernel launch");
    return TL_SUCCESS;
}

// Number of clusters of CL CTAs that can be resident at once with this shared-memory size (cached).
template <int KIND, typename TD, int CL>
int max_clusters(size_t smem)
{
    static std::mutex mu;
    static std::map<size_t, int> cache;
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(smem);
    if (it != cache.end()) return it->second;
    auto kern = tc_gemm_kernel<KIND, TD, CL, false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(CL, 1, 1);
    cfg.blockDim = dim3(kTcThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 0;
    }
    cache[smem] = n;
    return n;
}

}  // namespace tc
}  // namespace tl
