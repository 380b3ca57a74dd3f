/*
 * tensilelite.h -- C ABI of the GB300 (sm_103a) GEMM library.
 *
 * D = alpha * op(A) * op(B) + beta * C, column-major (BLAS) storage, FP32 accumulation.
 *
 * This boundary replaces TensileLite's C++ problem / solution / runtime surface for the GEMM path:
 *   - the problem + solution description T_GemmMfmaKernelParam (src/gemmMfmaKernelWriter.h:11-22)
 *     and its CLI flags (inc/ff_utils.h:347-361)                   -> tl_gemm_problem, tl_gemm_solution
 *   - GemmMfmaAsmSolution::generateKernel + StreamHip::Launch
 *     (src/gemmMfma.cpp:24-185, ff_gpu_src/ff_hip_runtime.cpp:278-320) -> tl_gemm
 *   - the kernel argument list D, C, A, B, alpha, beta, strides
 *     (src/gemmMfma.cpp:104-120)                                    -> tl_gemm arguments
 *   - checkKernelParameters (src/gemmMfmaKernelWriter.h:321-405)     -> tl_check_solution
 *   - GpuRuntimeBase DevMalloc/HostMalloc/MemCopy* (inc/ff_gpu.h:240-333),
 *     DataMem<T>::Sync2Dev/Sync2Hst (inc/ff_gpu.h:387-642)          -> tl_malloc ... tl_memcpy_*
 *   - E_ReturnState SUCCESS/RTN_WARN/RTN_ERR/RTN_FATAL (inc/ff_utils.h:44-50) -> tl_status 0..3
 *   - host converters cvtFP32toFP16/BF16 (inc/ff_utils.h:90-127)     -> tl_convert
 *   - the perf sweep test/perf_test.py:58-167                       -> tl_tune
 * Grouped GEMM, FP8, the bf16x3 FP32-accurate path and the device error norm have no reference
 * counterpart.
 *
 * Conventions: every call is asynchronous on the given CUDA stream (a cudaStream_t passed as
 * void*; NULL = legacy default stream) unless stated otherwise; nothing here calls exit(); every
 * call returns a tl_status and records a message retrievable with tl_last_error_string() (per
 * thread).  All device pointers are caller-owned.  A handle may be used from one host thread at a
 * time; separate handles are independent.
 */
#ifndef TENSILELITE_GB300_H
#define TENSILELITE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define TL_API __attribute__((visibility("default")))
#else
#define TL_API
#endif

/* Status codes.  0..3 keep the meaning of E_ReturnState (inc/ff_utils.h:44-50). */
typedef enum tl_status {
    TL_SUCCESS = 0,
    TL_WARN = 1,
    TL_ERR = 2,
    TL_FATAL = 3,
    TL_ERR_INVALID_ARG = 16,   /* bad size, stride, pointer or enum value */
    TL_ERR_UNSUPPORTED = 17,   /* legal problem that no kernel here implements */
    TL_ERR_TIMEOUT = 18,       /* a device-side wait ran out its limit (kernel returned early) */
    TL_ERR_CUDA = 19,          /* a CUDA runtime/driver call failed */
    TL_ERR_ALLOC = 20          /* device or host allocation failed */
} tl_status;

/* Element types.  1..3 are the reference's -d codes (src/gemmMfma.cpp:9, inc/ff_utils.h:347). */
typedef enum tl_dtype {
    TL_DTYPE_FP32 = 1,
    TL_DTYPE_FP16 = 2,
    TL_DTYPE_BF16 = 3,
    TL_DTYPE_FP8_E4M3 = 4
} tl_dtype;

/* op(X) = X (N) or X^T (T); column-major storage.  The reference kernel is TN only. */
typedef enum tl_op { TL_OP_N = 0, TL_OP_T = 1 } tl_op;

typedef enum tl_kernel {
    TL_KERNEL_AUTO = 0,     /* fp32 -> SIMT, fp16/bf16/fp8 -> TCGEN05 */
    TL_KERNEL_SIMT = 1,     /* CUDA-core FMA kernel, any input type, fp32 accumulation */
    TL_KERNEL_TCGEN05 = 2,  /* TMA -> smem ring -> tcgen05.mma (TMEM accumulator) -> epilogue */
    TL_KERNEL_BF16X3 = 3,   /* fp32 inputs split hi/lo into bf16, 3 tensor-core products */
    TL_KERNEL_BF16X6 = 4    /* fp32 inputs split into 3 bf16 pieces, 6 tensor-core products
                               (the terms of order <= 2^-16); FP32-class accuracy */
} tl_kernel;

/* Rounding of fp32 results into fp16/bf16 outputs.  TRUNCATE reproduces the reference's bf16
 * store (high 16 bits kept, src/gemmMfmaKernelWriter.h:1661-1665); fp16 is always RNE. */
typedef enum tl_rounding { TL_ROUND_RNE = 0, TL_ROUND_TRUNCATE = 1 } tl_rounding;

typedef struct tl_handle tl_handle;

/* One GEMM.  All sizes and strides are in elements.  op(A) is m x k, op(B) is k x n, C and D are
 * m x n with leading dimensions ldc/ldd.  Batch b uses A + b*stride_a (and likewise).  C may be
 * NULL when beta == 0 (then it is not read).  fp8 operands are dequantised by scale_a/scale_b:
 * D = alpha*scale_a*scale_b*op(A)op(B) + beta*C. */
typedef struct tl_gemm_problem {
    int32_t dtype_a, dtype_b, dtype_c, dtype_d;   /* tl_dtype; a == b, c == d */
    int32_t trans_a, trans_b;                     /* tl_op */
    int64_t m, n, k, batch;
    int64_t lda, ldb, ldc, ldd;
    int64_t stride_a, stride_b, stride_c, stride_d;
    float alpha, beta;
    float scale_a, scale_b;                       /* 0 is read as 1 */
    int32_t kernel;                               /* tl_kernel request */
    int32_t out_rounding;                         /* tl_rounding */
} tl_gemm_problem;

/* Solution (kernel configuration).  Field names keep the reference's vocabulary:
 *   macro_tile0/1  MT0 x MT1, the output tile along m / n (MT = mfma_mn*pttn*waves in the reference)
 *   depth_u        k per pipeline stage (loop_unroll / -u)
 *   stages         shared-memory ring depth (lds_buffer_num / -f)
 *   wave_tile0/1   SIMT: outputs per thread along m / n;  TCGEN05: ignored
 * TCGEN05: macro_tile1 is the tcgen05 M extent (128 on one SM, 256 on a CTA pair; problem n maps
 * to TMEM lanes) or 512 (two CTA pairs sharing the m-side operand through a TMA multicast load,
 * accepted only when A and B are memory of the current device, else TL_ERR_UNSUPPORTED; the
 * heuristic falls back to a CTA pair) and
 * macro_tile0 is the tcgen05 N extent (64, 128, 192 or 256 along m); depth_u is fixed by the
 * input type (64 for 16-bit, 128 for fp8: one 128-byte swizzle row).  split_k > 1 divides k
 * across CTAs and reduces through a device workspace owned by the handle.
 * promote_k > 0 (TCGEN05/BF16X3/BF16X6 with macro_tile0 == 128): the dominant product restarts its
 * tensor-core accumulation every promote_k elements of k and the chains are summed in fp32 on the
 * CUDA cores (tensor-core accumulation error grows with the chain length).
 * A single fp16/bf16 NN problem with beta == 0, k >= 2048 and split_k <= 1 runs on TCGEN05 as its
 * transposed product (D^T = B^T A^T, a TT problem, stored transposed into D): there the solution
 * describes that product, so macro_tile0 tiles n and macro_tile1 m (TL_NN_TRANSPOSE=0 turns this
 * off). */
typedef struct tl_gemm_solution {
    int32_t kernel;            /* resolved tl_kernel (never AUTO once filled in) */
    int32_t macro_tile0;
    int32_t macro_tile1;
    int32_t depth_u;
    int32_t stages;
    int32_t wave_tile0;
    int32_t wave_tile1;
    int32_t split_k;           /* >= 1 */
    int32_t raster;            /* tile rasterisation group width in tiles (0 = linear order) */
    int32_t ctas;              /* persistent CTAs (0 = one per SM) */
    int32_t promote_k;         /* k per tensor-core accumulation chain (0 = the whole k range) */
    int32_t tail_split;        /* split of a last, partial wave of tiles along k: 0 automatic,
                                  1 off, S >= 2 each of its tiles in S equal k-slices, -1 its
                                  k-blocks spread evenly over all workers (balanced) */
    int32_t debug_flags;       /* 0 for every real use; TL_DEBUG_SKIP_LOADS tests the timeout path */
    int32_t reserved[3];
} tl_gemm_solution;

/* debug_flags bits (tensor-core kernels).  TL_DEBUG_SKIP_LOADS: the TMA producer issues no copies,
 * so the MMA and epilogue waits run out their limit (tl_set_wait_timeout) and the call reports
 * TL_ERR_TIMEOUT through tl_device_status / tl_noalloc_status instead of computing D.  It exists
 * to test that a device wait that expires is reported and leaves the context usable; nothing is
 * issued that could still be in flight when the kernel returns. */
#define TL_DEBUG_SKIP_LOADS 1

/* ---- handles and errors --------------------------------------------------------------------- */

/* Create a handle on the current CUDA device (replaces RuntimeHip::GetInstance + SellectDevice,
 * ff_gpu_src/ff_hip_runtime.cpp:8-51; unlike the reference it is not a process singleton).  When the
 * environment variable TL_SOLUTIONS names a file written by tl_tune, its solutions for this device
 * are loaded (the tuned-solution database that replaces the reference's Tensile LibraryLogic yaml,
 * test/work/tensile tune). */
TL_API tl_status tl_init(tl_handle** handle);
/* A planning handle for a described device, made without any CUDA call and holding no device
 * memory: sm_count SMs, smem_optin bytes of opt-in shared memory per block, and clusters4 clusters
 * of four CTAs (one per SM) resident at once (0: sm_count / 4; a GB300 runs 36 on its 152 SMs).
 * Only tl_default_solution, tl_check_solution, tl_device_info (compute capability 10.3),
 * tl_load_solutions, tl_launch_count, tl_set_wait_timeout and tl_destroy accept it; calls that launch,
 * allocate or time work return TL_ERR_INVALID_ARG.  For offline planning and tests on hosts without
 * a GPU; no counterpart in the reference (its solver needs the device). */
TL_API tl_status tl_init_host(int sm_count, size_t smem_optin, int clusters4, tl_handle** handle);
TL_API tl_status tl_destroy(tl_handle* handle);
/* Message of the last failing call on this host thread ("" if none). */
TL_API const char* tl_last_error_string(void);
TL_API const char* tl_status_string(tl_status status);
/* Library version as major*10000 + minor*100 + patch. */
TL_API int tl_version(void);
/* Device properties the library keyed its choices on. */
TL_API tl_status tl_device_info(tl_handle* handle, int* sm_count, int* cc_major, int* cc_minor,
                                size_t* smem_per_block_optin);

/* ---- problems and solutions ----------------------------------------------------------------- */

/* Fill a problem with the defaults of a dense single-batch GEMM: lda/ldb/ldc/ldd = the minimal
 * column-major leading dimensions, alpha = 1, beta = 0, scales = 1, kernel = AUTO, RNE. */
TL_API tl_status tl_problem_init(tl_gemm_problem* problem, tl_dtype dtype_ab, tl_dtype dtype_cd,
                                 tl_op trans_a, tl_op trans_b, int64_t m, int64_t n, int64_t k);
/* Heuristic solution for a problem (no timing).  Replaces GemmMfmaSolver::generateSolver. */
TL_API tl_status tl_default_solution(tl_handle* handle, const tl_gemm_problem* problem,
                                     tl_gemm_solution* solution);
/* Legality of a solution for a problem (tile shape, smem/TMEM budget, alignment, k split);
 * mirrors checkKernelParameters.  TL_SUCCESS or TL_ERR_UNSUPPORTED/INVALID_ARG with a message. */
TL_API tl_status tl_check_solution(tl_handle* handle, const tl_gemm_problem* problem,
                                   const tl_gemm_solution* solution);

/* ---- GEMM ----------------------------------------------------------------------------------- */

/* D = alpha*op(A)*op(B) + beta*C on `stream`.  solution == NULL picks the tuned solution cached in
 * the handle for this problem, else the heuristic one.  D must not alias A, B or C unless D == C
 * with ldc == ldd (in-place beta update). */
TL_API tl_status tl_gemm(tl_handle* handle, const tl_gemm_problem* problem,
                         const tl_gemm_solution* solution, void* D, const void* C, const void* A,
                         const void* B, void* stream);

/* Time candidate solutions on the given buffers (D is overwritten) and return the fastest in
 * `best`; the result is cached in the handle and, if `cache_path` is non-NULL, merged into that
 * JSON file keyed by device and problem.  A candidate whose launches report a device error (a
 * bounded wait that ran out) is dropped, never returned or cached.  When D == C with beta != 0 the
 * candidates write a scratch output instead, so C is left intact.  Synchronous.  Replaces
 * test/perf_test.py:58-167. */
TL_API tl_status tl_tune(tl_handle* handle, const tl_gemm_problem* problem, void* D, const void* C,
                         const void* A, const void* B, int max_candidates, int reps,
                         const char* cache_path, tl_gemm_solution* best, float* best_ms);
/* ---- fused epilogue ------------------------------------------------------------------------------ */

/* Beyond alpha/beta: the reference fuses the beta*C update into its kernel's store
 * (src/gemmMfmaKernelWriter.h:1822-1906); tl_gemm_ex fuses a per-row bias, an activation and an
 * amax reduction the same way:  D = act(alpha*op(A)*op(B) + beta*C + bias[i])  for every element
 * (i, j) of the m x n output (bias broadcast along n: for a row-major Y = X*W viewed as
 * column-major, one value per output feature).  When amax is set, max |D| over the computed values
 * (before rounding to the output type) is atomically maxed into *amax (device float; initialise
 * it, e.g. to 0, before the call) -- the scale input of a following FP8 quantisation.  Tensor-core
 * kernels only (TL_ERR_UNSUPPORTED for the CUDA-core kernel). */
typedef enum tl_activation {
    TL_ACT_NONE = 0,
    TL_ACT_RELU = 1,
    TL_ACT_GELU = 2,   /* tanh approximation: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) */
    TL_ACT_SILU = 3    /* x / (1 + exp(-x)) */
} tl_activation;

typedef struct tl_epilogue {
    const void* bias;     /* NULL, or m device values of bias_dtype */
    int32_t bias_dtype;   /* TL_DTYPE_FP32, FP16 or BF16 */
    int32_t activation;   /* tl_activation */
    float* amax;          /* NULL, or a device float */
    float d_scale;        /* fp8 (E4M3) output: D = e4m3(d_scale * act(...)), round to nearest even,
                             saturating at +-448; 0 is read as 1; ignored for other outputs */
    int32_t reserved[3];
} tl_epilogue;

/* tl_gemm with a fused epilogue (epilogue == NULL: tl_gemm).
 * FP8 output (dtype_c = dtype_d = TL_DTYPE_FP8_E4M3, tensor-core kernels, beta == 0): the epilogue
 * quantises D = e4m3(d_scale * act(alpha*op(A)*op(B) + bias)); amax, when set, receives the max |.|
 * of the values before d_scale -- what the next step's scale is computed from.  tl_gemm with an fp8
 * output is the same with no bias, no activation and d_scale 1. */
TL_API tl_status tl_gemm_ex(tl_handle* handle, const tl_gemm_problem* problem, const tl_epilogue* epilogue,
                            const tl_gemm_solution* solution, void* D, const void* C, const void* A, const void* B,
                            void* stream);

/* ---- Tensile replacement-kernel entry ----------------------------------------------------------- */

/* The argument buffer of the reference's Tensile-layout kernel (`-t 1`, src/gemmMfma.cpp:70-103;
 * offsets by the kernel's argument table, src/gemmMfmaKernelWriter.h:321-338): 148 bytes, packed
 * with natural alignment as below.  The kernel is Tensile's Cijk_Alik_Bljk (TN, column-major):
 * D[i + j*stride_d0 + b*stride_d1] = alpha * sum_l A[l + i*stride_a0 + b*stride_a1] *
 * B[l + j*stride_b0 + b*stride_b1] + beta * C[...], with i < sizes_free0, j < sizes_free1,
 * b < sizes_free2, l < sizes_sum0.  alpha/beta are fp32 bits, or an fp16 value in the low half for
 * the HBH kernel.  The launch-geometry fields (stagger, work-group counts, magic numbers) are
 * Tensile's own and are ignored. */
#define TL_TENSILE_KERNARG_BYTES 148
typedef struct tl_tensile_kernarg {
    uint64_t size_c, size_a, size_b;   /* elements of each buffer (0: unchecked) */
    void* d;
    const void* c;
    const void* a;
    const void* b;
    uint32_t alpha_bits, beta_bits;
    uint32_t stride_d0, stride_d1, stride_c0, stride_c1, stride_a0, stride_a1, stride_b0, stride_b1;
    uint32_t sizes_free0, sizes_free1, sizes_free2, sizes_sum0;
    uint32_t orig_stagger_u_iter, num_work_groups0, num_work_groups1, magic_number_problem_num_group_tiles0,
        grid_num_work_groups0, num_full_blocks, wgm_remainder1, magic_number_wgm_remainder1, padding;
} tl_tensile_kernarg;

/* Run the GEMM a Tensile-layout kernel launch describes: `kernel_name` is
 * Cijk_Alik_Bljk_{SB,HBH,BBH}[_...] (the names of src/gemmMfmaKernelWriter.h:376-378: fp32, fp16,
 * bf16 operands and output; the bf16 output truncates as that kernel does), `kernarg` the argument
 * buffer (at least TL_TENSILE_KERNARG_BYTES).  Asynchronous on `stream`, through tl_gemm with the
 * handle's tuned or heuristic solution.  Replaces launching the generated kernel with Tensile's
 * argument buffer (run_feifei_rpk.py:25-35 drives it from Tensile's client). */
TL_API tl_status tl_tensile_launch(tl_handle* handle, const char* kernel_name, const void* kernarg,
                                   size_t kernarg_bytes, void* stream);

/* Load tuned solutions from a JSON file written by tl_tune into the handle's cache. */
TL_API tl_status tl_load_solutions(tl_handle* handle, const char* cache_path, int* loaded);

/* The tcgen05 GEMM (split-k included) without any allocation, for callers that cannot call
 * cudaMalloc: an application that owns all device memory through its own pool, a latency-critical
 * path where an allocation (which may synchronise the device) is not acceptable, or a caller with no
 * tl_handle (creating one allocates).  No counterpart in the reference.  Split-k partials, tile
 * counters and the error word live in one static device array of 64 MiB per device (held until the
 * process exits); problems whose workspace exceeds it are refused with TL_ERR_UNSUPPORTED.  All calls
 * share that array: each clears the parts it uses, and calls that overlap on the GPU race.  The
 * first call on a device looks the array up with that device current -- make it before any stream
 * capture.  The call runs on the caller's current device and context (runtime API) and never
 * changes them.  fp16/bf16/fp8 operands (TCGEN05 only); solution == NULL uses the heuristic.  A
 * bounded device wait that runs out is recorded in the array's error word: read it with
 * tl_noalloc_status. */
TL_API tl_status tl_gemm_noalloc(const tl_gemm_problem* problem, const tl_gemm_solution* solution, void* D,
                                 const void* C, const void* A, const void* B, void* stream);
/* Synchronise `stream` and read, then clear, the error word of the last tl_gemm_noalloc call on the
 * current device (each call clears it when it starts): TL_SUCCESS, or TL_ERR_TIMEOUT when a device
 * wait of that call ran out and D is not valid.  Allocates nothing.  No counterpart in the
 * reference (its launches report through E_ReturnState, inc/ff_utils.h:44-50). */
TL_API tl_status tl_noalloc_status(void* stream);

/* ---- grouped GEMM (one persistent launch over many independent problems) ---------------------- */

typedef struct tl_grouped_plan tl_grouped_plan;

/* Build a plan: validates every problem (all must share dtypes and trans flags; sizes, leading
 * dimensions, alpha/beta and pointers may differ), encodes their TMA descriptors and uploads the
 * problem table.  Synchronous.  solution == NULL uses the heuristic tile for the group. */
TL_API tl_status tl_grouped_plan_create(tl_handle* handle, const tl_gemm_problem* problems,
                                        int count, void* const* D, const void* const* C,
                                        const void* const* A, const void* const* B,
                                        const tl_gemm_solution* solution, tl_grouped_plan** plan);
/* Launch the plan's single persistent kernel on `stream`; capturable in a CUDA graph. */
TL_API tl_status tl_grouped_plan_launch(tl_grouped_plan* plan, void* stream);
TL_API tl_status tl_grouped_plan_destroy(tl_grouped_plan* plan);
/* Total FLOPs (2*m*n*k summed) and tile count of a plan. */
TL_API tl_status tl_grouped_plan_info(const tl_grouped_plan* plan, double* flops, int64_t* tiles,
                                      tl_gemm_solution* solution);
/* create + launch + destroy (the plan is released after the stream drains).  Synchronous. */
TL_API tl_status tl_gemm_grouped(tl_handle* handle, const tl_gemm_problem* problems, int count,
                                 void* const* D, const void* const* C, const void* const* A,
                                 const void* const* B, void* stream);
/* Tile-shape autotuner for a group: times each candidate with the plan's launch and returns the
 * fastest.  Synchronous; D buffers are overwritten. */
TL_API tl_status tl_tune_grouped(tl_handle* handle, const tl_gemm_problem* problems, int count,
                                 void* const* D, const void* const* C, const void* const* A,
                                 const void* const* B, int reps, tl_gemm_solution* best,
                                 float* best_ms);

/* ---- CUDA graphs ---------------------------------------------------------------------------- */

typedef struct tl_graph tl_graph;
/* Capture one plan launch on `stream` into an executable graph. */
TL_API tl_status tl_graph_capture_grouped(tl_grouped_plan* plan, void* stream, tl_graph** graph);
/* Capture one tl_gemm call (solution resolved at capture time) into an executable graph. */
TL_API tl_status tl_graph_capture_gemm(tl_handle* handle, const tl_gemm_problem* problem,
                                       const tl_gemm_solution* solution, void* D, const void* C,
                                       const void* A, const void* B, void* stream, tl_graph** graph);
TL_API tl_status tl_graph_launch(tl_graph* graph, void* stream);
TL_API tl_status tl_graph_destroy(tl_graph* graph);

/* ---- fp8 and split helpers ------------------------------------------------------------------ */

/* amax = max|x| over n elements of src (fp32/fp16/bf16), then dst = e4m3(x * 448/amax)
 * (round-to-nearest-even, saturating).  *scale_out (device float, optional) receives the
 * dequantisation factor amax/448 (1 when amax == 0).  amax_out (device float, optional). */
TL_API tl_status tl_quantize_fp8(tl_handle* handle, tl_dtype src_dtype, const void* src, int64_t n,
                                 void* dst_e4m3, float* scale_out_dev, float* amax_out_dev,
                                 void* stream);
/* hi = bf16_rne(x), lo = bf16_rne(x - hi) for n fp32 values (the bf16x3 split). */
TL_API tl_status tl_split_bf16x2(tl_handle* handle, const float* src, int64_t n, void* hi, void* lo,
                                 void* stream);

/* ---- verification --------------------------------------------------------------------------- */

/* On-device FP64 error norms of D (m x n, ldd, dtype_d) against a reference R (m x n, ldr, fp64):
 * out[0] = max|d - r|, out[1] = max|r|, out[2] = max |d - r| / w where w (optional, fp64, ldr)
 * holds the componentwise weights sum_k |a||b| (0 if w == NULL).  out is a host array of 3;
 * synchronous.  FP64 is used only in this reduction, never in a contraction. */
TL_API tl_status tl_error_norms(tl_handle* handle, tl_dtype dtype_d, const void* D, int64_t ldd,
                                const double* R, const double* W, int64_t ldr, int64_t m, int64_t n,
                                double out[3], void* stream);

/* ---- buffers (DataMem / GpuRuntimeBase counterparts) ---------------------------------------- */

TL_API tl_status tl_malloc(void** dev_ptr, size_t bytes);
TL_API tl_status tl_free(void* dev_ptr);
TL_API tl_status tl_host_malloc(void** host_ptr, size_t bytes);   /* pinned */
TL_API tl_status tl_host_free(void* host_ptr);
TL_API tl_status tl_memcpy_h2d(void* dst, const void* src, size_t bytes, void* stream);
TL_API tl_status tl_memcpy_d2h(void* dst, const void* src, size_t bytes, void* stream);
TL_API tl_status tl_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream);
TL_API tl_status tl_memset(void* dev_ptr, int value, size_t bytes, void* stream);
TL_API tl_status tl_stream_create(void** stream);
TL_API tl_status tl_stream_destroy(void* stream);
TL_API tl_status tl_stream_synchronize(void* stream);
/* Device-side fill with the reference's deterministic patterns (InitRealData,
 * ff_gpu_src/ff_gpu.cpp:110-148): code 2.4 -> idx % 7, -2.4 -> -(idx % 11), ...; count elements
 * of dtype at dst, flat index idx. */
TL_API tl_status tl_fill_pattern(tl_dtype dtype, void* dst, int64_t count, float code, void* stream);
/* Host converters: fp32 -> dtype bits with the given rounding (inc/ff_utils.h:90-127 behaviour
 * for fp16; bf16 TRUNCATE is the reference's cvtFP32toBF16). */
TL_API tl_status tl_convert_host(const float* src, int64_t n, tl_dtype dtype, tl_rounding rounding,
                                 void* dst);

/* ---- timing (CUDA events on a stream) -------------------------------------------------------- */

typedef struct tl_timer tl_timer;
TL_API tl_status tl_timer_create(tl_timer** timer);
TL_API tl_status tl_timer_start(tl_timer* timer, void* stream);
TL_API tl_status tl_timer_stop(tl_timer* timer, void* stream);
TL_API tl_status tl_timer_elapsed_ms(tl_timer* timer, float* ms);   /* synchronises the stop */
TL_API tl_status tl_timer_destroy(tl_timer* timer);

/* Per-launch kernel timing.  The reference times every kernel launch with a start/stop event pair
 * and blocks until the stop (StreamHip::Launch, ff_gpu_src/ff_hip_runtime.cpp:278-320, read back as
 * kernelExeTime in SolutionCtrlBase::run_comb_kernel, ff_gpu_src/ff_gpu_test_fw.cpp:24-52).  Here,
 * while enabled, an event pair is recorded on the launching stream around each GEMM kernel launch
 * (tl_gemm's tensor-core or CUDA-core kernel, a grouped plan's launch; not the split/quantise
 * pre-passes) without blocking; tl_kernel_timing waits for the recorded launches and returns the
 * summed kernel time and the number of timed launches (reset != 0 clears both afterwards).
 * Launches into a stream that is being captured are not timed. */
TL_API tl_status tl_set_kernel_timing(tl_handle* handle, int enable);
TL_API tl_status tl_kernel_timing(tl_handle* handle, double* total_ms, int64_t* launches, int reset);

/* Number of library kernel launches issued through this handle since creation. */
TL_API tl_status tl_launch_count(tl_handle* handle, int64_t* launches);

/* Synchronise `stream` and read (then clear) the handle's device error word.  Kernels that ran
 * out a bounded wait set it and return early instead of hanging: TL_ERR_TIMEOUT.  A pending CUDA
 * error gives TL_ERR_CUDA. */
TL_API tl_status tl_device_status(tl_handle* handle, void* stream);
/* Limit of every device-side wait, in milliseconds (default 4000; also env TL_WAIT_TIMEOUT_MS). */
TL_API tl_status tl_set_wait_timeout(tl_handle* handle, uint32_t ms);

/* Device timeline of the tensor-core kernel, the counterpart of the reference's per-wave thread
 * trace (test/ttrace, read with s_memtime stamps in its kernels).  While a buffer is set, every
 * tensor-core GEMM launched through the handle writes, for each CTA, TL_TRACE_SLOTS 64-bit words
 * at [cta * TL_TRACE_SLOTS]: the SM cycle counter (%clock64) at the events below, for the CTA's
 * first tile, plus the global nanosecond timer at entry and exit and the SM id.  A launch whose
 * grid needs more words than `bytes` holds records nothing.  NULL (or 0 bytes) switches it off.
 * The buffer is device memory the caller owns; slots of events a CTA does not reach are left as
 * they were (fill the buffer with zeros first). */
#define TL_TRACE_SLOTS 16
enum {
    TL_TRACE_ENTRY = 0,        /* kernel entry */
    TL_TRACE_ENTRY_NS = 1,     /* %globaltimer at entry */
    TL_TRACE_SETUP = 2,        /* barriers initialised, TMEM allocated, CTAs of the cluster in step */
    TL_TRACE_DEP = 3,          /* the previous grid in the stream has completed (programmatic launch) */
    TL_TRACE_LOAD_FIRST = 4,   /* producer: starts issuing the first tile's TMA loads */
    TL_TRACE_LOAD_LAST = 5,    /* producer: first tile's last TMA load issued */
    TL_TRACE_MMA_FIRST = 6,    /* MMA warp: first tile's first stage landed */
    TL_TRACE_MMA_LAST = 7,     /* MMA warp: first tile's last MMA committed */
    TL_TRACE_ACC_READY = 8,    /* epilogue: first tile's accumulator ready */
    TL_TRACE_STORED = 9,       /* epilogue: first tile's output (or split-k partial) written */
    TL_TRACE_REDUCED = 10,     /* epilogue: split-k reduction of the first tile finished */
    TL_TRACE_EPI_END = 11,     /* epilogue: every tile done */
    TL_TRACE_EXIT = 12,        /* TMEM released, CTA about to exit */
    TL_TRACE_EXIT_NS = 13,     /* %globaltimer at exit */
    TL_TRACE_SMID = 14,        /* the SM the CTA ran on */
    TL_TRACE_TILES = 15        /* work units the CTA processed */
};
TL_API tl_status tl_set_trace(tl_handle* handle, void* device_buffer, int64_t bytes);

#ifdef __cplusplus
}
#endif
#endif /* TENSILELITE_GB300_H */
