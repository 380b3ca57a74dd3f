// aux_kernels.cu -- the memory-bound helpers around the GEMM:
//   split_bf16       fp32 -> 2 or 3 bf16 pieces for the FP32-accurate bf16x3 / bf16x6 products
//   amax / quant     per-tensor amax and E4M3 quantisation (scale = 448 / amax)
//   error_norms      FP64 reduction of max|d - r|, max|r| and the componentwise ratio
//   fill_pattern     the reference's deterministic InitRealData codes, on the device
//   scale_c          D = beta * C (the k == 0 GEMM)
// All are grid-stride kernels over 16-byte vectors where the layout allows; grids are multiples of
// the SM count.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "tl_internal.h"

namespace tl {
namespace {

int grid_for(int64_t n, int per_thread, int threads)
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 132;
    }
    int64_t want = (n + static_cast<int64_t>(per_thread) * threads - 1) / (static_cast<int64_t>(per_thread) * threads);
    const int64_t cap = static_cast<int64_t>(sms) * 8;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return static_cast<int>(want);
}

__device__ __forceinline__ float load_as_float(int dtype, const void* p, int64_t i)
{
    switch (dtype) {
    case TL_DTYPE_FP32: return static_cast<const float*>(p)[i];
    case TL_DTYPE_FP16: return __half2float(static_cast<const __half*>(p)[i]);
    case TL_DTYPE_BF16: return __bfloat162float(static_cast<const __nv_bfloat16*>(p)[i]);
    case TL_DTYPE_FP8_E4M3: return static_cast<float>(static_cast<const __nv_fp8_e4m3*>(p)[i]);
    default: return 0.f;
    }
}

__device__ __forceinline__ void store_from_float(int dtype, int trunc, void* p, int64_t i, float v)
{
    switch (dtype) {
    case TL_DTYPE_FP32: static_cast<float*>(p)[i] = v; break;
    case TL_DTYPE_FP16: static_cast<__half*>(p)[i] = __float2half_rn(v); break;
    case TL_DTYPE_BF16:
        if (trunc) static_cast<uint16_t*>(p)[i] = static_cast<uint16_t>(__float_as_uint(v) >> 16);
        else static_cast<__nv_bfloat16*>(p)[i] = __float2bfloat16_rn(v);
        break;
    case TL_DTYPE_FP8_E4M3:
        static_cast<uint8_t*>(p)[i] = static_cast<uint8_t>(__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3));
        break;
    default: break;
    }
}

// ---- split-precision pieces -------------------------------------------------------------------------
// p0 = bf16(x), p1 = bf16(x - p0), p2 = bf16(x - p0 - p1); every subtraction is exact in fp32 (the
// residual of a rounding is representable), so x = p0 + p1 + p2 + O(2^-24 |x|).
template <int NP>
__device__ __forceinline__ void split_pieces(float x, uint16_t (&o)[3])
{
    float r = x;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const __nv_bfloat16 b = __float2bfloat16_rn(r);
        o[i] = __bfloat16_as_ushort(b);
        r = r - __bfloat162float(b);
    }
}

template <int NP>
__global__ void split_kernel(const float* __restrict__ src, int64_t rows, int64_t cols, int64_t ld, int64_t batch,
                             int64_t bs, uint16_t* __restrict__ p0, uint16_t* __restrict__ p1,
                             uint16_t* __restrict__ p2)
{
    // element e of the logical rows x cols x batch block lives at b*bs + c*ld + r
    const int64_t total = rows * cols * batch;
    const bool dense = (ld == rows) && (batch == 1 || bs == rows * cols);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    uint16_t* out[3] = {p0, p1, p2};
    bool vec = dense && (reinterpret_cast<uintptr_t>(src) & 15) == 0;
#pragma unroll
    for (int i = 0; i < NP; ++i) vec = vec && (reinterpret_cast<uintptr_t>(out[i]) & 7) == 0;
    if (vec) {
        const int64_t n4 = total / 4;
        for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n4; i += stride) {
            const float4 v = reinterpret_cast<const float4*>(src)[i];
            uint16_t q[4][3];
            split_pieces<NP>(v.x, q[0]);
            split_pieces<NP>(v.y, q[1]);
            split_pieces<NP>(v.z, q[2]);
            split_pieces<NP>(v.w, q[3]);
#pragma unroll
            for (int pc = 0; pc < NP; ++pc)
                reinterpret_cast<uint2*>(out[pc])[i] = make_uint2(q[0][pc] | (uint32_t(q[1][pc]) << 16),
                                                                  q[2][pc] | (uint32_t(q[3][pc]) << 16));
        }
        for (int64_t i = n4 * 4 + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total; i += stride) {
            uint16_t q[3];
            split_pieces<NP>(src[i], q);
#pragma unroll
            for (int pc = 0; pc < NP; ++pc) out[pc][i] = q[pc];
        }
        return;
    }
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total; e += stride) {
        const int64_t r = e % rows;
        const int64_t c = (e / rows) % cols;
        const int64_t b = e / (rows * cols);
        const int64_t off = b * bs + c * ld + r;
        uint16_t q[3];
        split_pieces<NP>(src[off], q);
#pragma unroll
        for (int pc = 0; pc < NP; ++pc) out[pc][off] = q[pc];
    }
}

// ---- fp8 ----------------------------------------------------------------------------------------------
__global__ void amax_kernel(int dtype, const void* __restrict__ src, int64_t n, float* amax)
{
    float m = 0.f;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
        m = fmaxf(m, fabsf(load_as_float(dtype, src, i)));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) atomicMax(reinterpret_cast<unsigned int*>(amax), __float_as_uint(m));
    }
}

__global__ void quant_kernel(int dtype, const void* __restrict__ src, int64_t n, const float* __restrict__ amax,
                             uint8_t* __restrict__ dst, float* scale_out)
{
    const float a = *amax;
    const float s = a > 0.f ? 448.0f / a : 1.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0 && scale_out) *scale_out = a > 0.f ? a / 448.0f : 1.0f;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride) {
        const float x = load_as_float(dtype, src, i) * s;
        dst[i] = static_cast<uint8_t>(__nv_cvt_float_to_fp8(x, __NV_SATFINITE, __NV_E4M3));
    }
}

// ---- error norms ------------------------------------------------------------------------------------
__device__ __forceinline__ void atomic_max_nonneg(double* p, double v)
{
    atomicMax(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(__double_as_longlong(v)));
}

__global__ void norms_kernel(int dtype, const void* __restrict__ D, int64_t ldd, const double* __restrict__ R,
                             const double* __restrict__ W, int64_t ldr, int64_t m, int64_t n, double* out)
{
    double md = 0.0, mr = 0.0, mc = 0.0;
    const int64_t total = m * n;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total; e += stride) {
        const int64_t i = e % m, j = e / m;
        const double d = static_cast<double>(load_as_float(dtype, D, i + j * ldd));
        const double r = R[i + j * ldr];
        const double diff = fabs(d - r);
        md = fmax(md, diff);
        mr = fmax(mr, fabs(r));
        if (W) {
            const double w = W[i + j * ldr];
            if (w > 0.0) mc = fmax(mc, diff / w);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
        mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        mc = fmax(mc, __shfl_xor_sync(0xffffffffu, mc, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_nonneg(out + 0, md);
        atomic_max_nonneg(out + 1, mr);
        atomic_max_nonneg(out + 2, mc);
    }
}

// ---- patterns ------------------------------------------------------------------------------------
// InitRealData codes (ff_gpu_src/ff_gpu.cpp:110-148) that depend on the flat index only.
__global__ void fill_kernel(int dtype, void* dst, int64_t count, float code)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count; i += stride) {
        const uint32_t idx = static_cast<uint32_t>(i);
        float v;
        if (code == 0.5f || code == 0.0f) v = 0.f;
        else if (code == 1.0f) v = 1.0f;
        else if (code == 2.0f) v = static_cast<float>(idx);
        else if (code == 2.1f) v = 0.01f * static_cast<float>(idx % 1137u);
        else if (code == 2.3f) v = 0.1f * static_cast<float>(idx % 17u);
        else if (code == 2.4f) v = static_cast<float>(idx % 7u);
        else if (code == -1.0f) v = -1.0f;
        else if (code == -2.0f) v = -static_cast<float>(idx);
        else if (code == -2.1f) v = -0.01f * static_cast<float>(idx % 1137u);
        else if (code == -2.3f) v = -0.1f * static_cast<float>(idx % 17u);
        else if (code == -2.4f) v = -static_cast<float>(idx % 11u);
        else v = code;
        if (dtype == TL_DTYPE_FP8_E4M3)
            static_cast<uint8_t*>(dst)[i] = static_cast<uint8_t>(__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3));
        else
            store_from_float(dtype, 0, dst, i, v);
    }
}

__global__ void scale_c_kernel(int dtype, int trunc, void* D, int64_t ldd, int64_t sd, const void* C, int64_t ldc,
                               int64_t sc, int64_t M, int64_t N, int64_t batch, float beta)
{
    const int64_t total = M * N * batch;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total; e += stride) {
        const int64_t i = e % M, j = (e / M) % N, b = e / (M * N);
        float v = 0.f;
        if (beta != 0.f && C) v = beta * load_as_float(dtype, C, b * sc + i + j * ldc);
        store_from_float(dtype, trunc, D, b * sd + i + j * ldd, v);
    }
}

tl_status check_launch(const char* what, int64_t* launches)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (launches) ++*launches;
    return TL_SUCCESS;
}

}  // namespace

tl_status aux_split_bf16(const float* src, int64_t rows, int64_t cols, int64_t ld, int64_t batch,
                         int64_t batch_stride, uint16_t* p0, uint16_t* p1, uint16_t* p2, cudaStream_t s,
                         int64_t* launches)
{
    const int64_t total = rows * cols * batch;
    if (total == 0) return TL_SUCCESS;
    const int grid = grid_for(total, 8, 256);
    if (p2) split_kernel<3><<<grid, 256, 0, s>>>(src, rows, cols, ld, batch, batch_stride, p0, p1, p2);
    else split_kernel<2><<<grid, 256, 0, s>>>(src, rows, cols, ld, batch, batch_stride, p0, p1, nullptr);
    return check_launch("split_kernel", launches);
}

tl_status aux_amax(int src_dtype, const void* src, int64_t n, float* amax_dev, cudaStream_t s, int64_t* launches)
{
    TL_CUDA_TRY(cudaMemsetAsync(amax_dev, 0, sizeof(float), s));
    if (n == 0) return TL_SUCCESS;
    amax_kernel<<<grid_for(n, 8, 256), 256, 0, s>>>(src_dtype, src, n, amax_dev);
    return check_launch("amax_kernel", launches);
}

tl_status aux_quant_e4m3(int src_dtype, const void* src, int64_t n, const float* amax_dev, uint8_t* dst,
                         float* scale_out_dev, cudaStream_t s, int64_t* launches)
{
    quant_kernel<<<grid_for(n > 0 ? n : 1, 8, 256), 256, 0, s>>>(src_dtype, src, n, amax_dev, dst, scale_out_dev);
    return check_launch("quant_kernel", launches);
}

tl_status aux_error_norms(int dtype_d, const void* D, int64_t ldd, const double* R, const double* W, int64_t ldr,
                          int64_t m, int64_t n, double* out_dev, cudaStream_t s, int64_t* launches)
{
    TL_CUDA_TRY(cudaMemsetAsync(out_dev, 0, 3 * sizeof(double), s));
    if (m * n == 0) return TL_SUCCESS;
    norms_kernel<<<grid_for(m * n, 8, 256), 256, 0, s>>>(dtype_d, D, ldd, R, W, ldr, m, n, out_dev);
    return check_launch("norms_kernel", launches);
}

tl_status aux_fill_pattern(int dtype, void* dst, int64_t count, float code, cudaStream_t s, int64_t* launches)
{
    if (count == 0) return TL_SUCCESS;
    fill_kernel<<<grid_for(count, 8, 256), 256, 0, s>>>(dtype, dst, count, code);
    return check_launch("fill_kernel", launches);
}

tl_status aux_scale_c(int out_dtype, int out_trunc, void* D, int64_t ldd, int64_t sd, const void* C, int64_t ldc,
                      int64_t sc, int64_t M, int64_t N, int64_t batch, float beta, cudaStream_t s,
                      int64_t* launches)
{
    const int64_t total = M * N * batch;
    if (total == 0) return TL_SUCCESS;
    scale_c_kernel<<<grid_for(total, 8, 256), 256, 0, s>>>(out_dtype, out_trunc, D, ldd, sd, C, ldc, sc, M, N, batch,
                                                           beta);
    return check_launch("scale_c_kernel", launches);
}

}  // namespace tl
