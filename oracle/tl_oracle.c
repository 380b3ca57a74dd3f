/*
 * tl_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of TensileLite's host-side arithmetic for the GEMM path.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library, and only as the
 * checker or as the timed CPU baseline.  The product (libtensilelite_gb300.so) never links it.
 *
 * What is restated, with the reference location each function follows:
 *   orc_f32_to_f16          inc/ff_utils.h:90-111  cvtFP32toFP16  (IEEE round-to-nearest-even,
 *                                                  NaN -> quiet NaN 0x7e00 | sign, overflow -> inf)
 *   orc_ref_f16_to_f32      inc/ff_utils.h:112-118 cvtFP16toFP32 as the reference executes it:
 *                                                  pow(1.0, +-112) == 1, so subnormal halves decode
 *                                                  to 2^-15 * (1 + m/1024) and inf/NaN decode to
 *                                                  2^16 * (1 + m/1024).  Normal values are exact.
 *   orc_f32_to_bf16_trunc   inc/ff_utils.h:119-122 cvtFP32toBF16 (keeps the high 16 bits)
 *   orc_bf16_to_f32         inc/ff_utils.h:123-127 cvtBF16toFP32
 *   orc_init_pattern        ff_gpu_src/ff_gpu.cpp:110-148 InitRealData (the integer codes 2.4 / -2.4
 *                                                  used by src/gemmMfma.cpp:231-235, and friends)
 *   orc_gemm_ref_f32        src/gemmMfma.cpp:313-346 GemmMfmaProblem::cpuCompute: float accumulator,
 *                                                  k ascending, t = alpha*t + beta*c, no FMA
 *                                                  contraction (build with -ffp-contract=off; the
 *                                                  reference is built -O0, build.py:34).
 * Additional oracles that have no reference counterpart but are fixed by the task:
 *   orc_f16_to_f32          exact IEEE half decode (for FP64 error metrics)
 *   orc_f32_to_bf16_rne     IEEE round-to-nearest-even bf16 (how seeded inputs are cast)
 *   orc_f32_to_e4m3 / orc_e4m3_to_f32   OCP FP8 E4M3 (fn variant: no inf, NaN = 0x7f/0xff,
 *                                       max finite 448), round-to-nearest-even, saturating
 *   orc_gemm_f64            the same loop accumulated in double (FP64 host oracle)
 *
 * The reference's kernel is TN only (A stored K-contiguous per m, B stored K-contiguous per n).
 * The GEMM oracles here take BLAS column-major op(A)/op(B) flags and index through them, which is
 * the same loop for trans_a = 1, trans_b = 0 (the reference's TN).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_API __attribute__((visibility("default")))

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* ---------------------------------------------------------------------------------------------
 * Converters
 * ------------------------------------------------------------------------------------------- */

/* fp32 -> fp16, round to nearest even.  Written from the IEEE 754 binary16 definition. */
ORC_API uint16_t orc_f32_to_f16(float f)
{
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t e = (x >> 23) & 0xffu;
    uint32_t man = x & 0x7fffffu;
    if (e == 0xffu)                           /* inf or NaN */
        return (uint16_t)(sign | 0x7c00u | (man ? 0x0200u : 0u));
    int32_t he = (int32_t)e - 127 + 15;       /* biased half exponent */
    if (he >= 31)                             /* certainly overflows */
        return (uint16_t)(sign | 0x7c00u);
    uint32_t full = man | 0x800000u;          /* 24-bit significand incl. hidden bit */
    if (e == 0) full = man;                   /* fp32 subnormal: far below half range */
    int32_t shift;                            /* right shift from the 24-bit significand */
    uint32_t base;
    if (he >= 1) { shift = 13; base = (uint32_t)he << 10; full &= 0x7fffffu; }
    else {                                    /* result is subnormal (or zero) in half */
        shift = 14 - he;                      /* 13 + (1 - he) */
        base = 0;
        if (shift > 31) return (uint16_t)sign;
    }
    uint32_t q = full >> shift;
    uint32_t rem = full & ((1u << shift) - 1u);
    uint32_t halfway = 1u << (shift - 1);
    uint32_t r = base + q;
    if (rem > halfway || (rem == halfway && (q & 1u))) r += 1u;  /* carry may bump exponent */
    if (r >= 0x7c00u) r = 0x7c00u;
    return (uint16_t)(sign | r);
}

/* The reference's fp16 -> fp32 decode, restated bit by bit (see header). */
ORC_API float orc_ref_f16_to_f32(uint16_t a)
{
    uint32_t sign = ((uint32_t)a & 0x8000u) << 16;
    uint32_t e = ((uint32_t)a >> 10) & 0x1fu;
    uint32_t man = (uint32_t)a & 0x3ffu;
    if (e == 0 && man == 0) return u2f(sign);
    /* the reference rebiases every non-zero input by +112 in the exponent field, after placing the
       5-bit exponent in the low bits of the fp32 exponent field; its 2^112 scale factor is 1 */
    uint32_t ef = e + 112u;
    return u2f(sign | (ef << 23) | (man << 13));
}

/* Exact IEEE binary16 decode. */
ORC_API float orc_f16_to_f32(uint16_t a)
{
    uint32_t sign = ((uint32_t)a & 0x8000u) << 16;
    uint32_t e = ((uint32_t)a >> 10) & 0x1fu;
    uint32_t man = (uint32_t)a & 0x3ffu;
    if (e == 0x1f) return u2f(sign | 0x7f800000u | (man << 13));
    if (e == 0) {
        float v = (float)man * 0x1p-24f;
        return sign ? -v : v;
    }
    return u2f(sign | ((e + 112u) << 23) | (man << 13));
}

ORC_API uint16_t orc_f32_to_bf16_trunc(float f) { return (uint16_t)(f2u(f) >> 16); }

ORC_API uint16_t orc_f32_to_bf16_rne(float f)
{
    uint32_t x = f2u(f);
    if ((x & 0x7f800000u) == 0x7f800000u && (x & 0x7fffffu))
        return (uint16_t)((x >> 16) | 0x0040u);           /* quiet NaN */
    uint32_t lsb = (x >> 16) & 1u;
    x += 0x7fffu + lsb;
    return (uint16_t)(x >> 16);
}

ORC_API float orc_bf16_to_f32(uint16_t b) { return u2f((uint32_t)b << 16); }

/* OCP FP8 E4M3 ("fn": 4 exponent bits, bias 7, 3 mantissa bits, no inf, NaN = S.1111.111).
 * Round to nearest even; values beyond 448 saturate to +-448 (satfinite); NaN -> 0x7f. */
ORC_API uint8_t orc_f32_to_e4m3(float f)
{
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 24) & 0x80u;
    if ((x & 0x7f800000u) == 0x7f800000u) {
        if (x & 0x7fffffu) return 0x7f;
        return (uint8_t)(sign | 0x7e);                     /* inf saturates */
    }
    float a = fabsf(f);
    if (a >= 464.0f) return (uint8_t)(sign | 0x7e);        /* >= midpoint(448, 480): saturate */
    /* scale into an integer grid: for exponent E (unbiased), step = 2^(E-3); subnormal step 2^-9 */
    int E;
    if (a < 0x1p-6f) E = -6;                                /* subnormal range uses step 2^-9 */
    else { frexpf(a, &E); E -= 1; }                         /* a in [2^E, 2^(E+1)) */
    float step = ldexpf(1.0f, E - 3);
    float q = a / step;                                     /* exact: power-of-two scale */
    float fl = floorf(q);
    float rem = q - fl;
    uint32_t qi = (uint32_t)fl;
    if (rem > 0.5f || (rem == 0.5f && (qi & 1u))) qi += 1u;
    /* rebuild bits: value = qi * step */
    if (qi == 0) return (uint8_t)sign;
    uint32_t bits;
    if (E == -6 && qi < 8) bits = qi;                       /* subnormal */
    else {
        if (qi >= 16) { qi >>= 1; E += 1; }                 /* rounding carried into next binade */
        if (E == -6 && qi < 8) bits = qi;
        else bits = ((uint32_t)(E + 7) << 3) | (qi & 7u);
    }
    if (bits > 0x7e) bits = 0x7e;
    return (uint8_t)(sign | bits);
}

ORC_API float orc_e4m3_to_f32(uint8_t v)
{
    uint32_t sign = v & 0x80u;
    uint32_t e = (v >> 3) & 0xfu;
    uint32_t m = v & 7u;
    float r;
    if (e == 0xf && m == 7) return u2f(0x7fc00000u | (sign << 24));
    if (e == 0) r = ldexpf((float)m, -9);
    else r = ldexpf((float)(8 + m), (int)e - 10);
    return sign ? -r : r;
}

/* Bulk forms over arrays (the tests and golden generators use these). */
ORC_API void orc_f32_to_f16_n(const float* x, uint16_t* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_f32_to_f16(x[i]); }
ORC_API void orc_f16_to_f32_n(const uint16_t* x, float* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_f16_to_f32(x[i]); }
ORC_API void orc_ref_f16_to_f32_n(const uint16_t* x, float* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_ref_f16_to_f32(x[i]); }
ORC_API void orc_f32_to_bf16_trunc_n(const float* x, uint16_t* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_f32_to_bf16_trunc(x[i]); }
ORC_API void orc_f32_to_bf16_rne_n(const float* x, uint16_t* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_f32_to_bf16_rne(x[i]); }
ORC_API void orc_bf16_to_f32_n(const uint16_t* x, float* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_bf16_to_f32(x[i]); }
ORC_API void orc_f32_to_e4m3_n(const float* x, uint8_t* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_f32_to_e4m3(x[i]); }
ORC_API void orc_e4m3_to_f32_n(const uint8_t* x, float* y, int64_t n)
{ for (int64_t i = 0; i < n; ++i) y[i] = orc_e4m3_to_f32(x[i]); }

/* ---------------------------------------------------------------------------------------------
 * Deterministic init patterns: InitRealData, ff_gpu_src/ff_gpu.cpp:110-148.
 * Buffer is dim0 (fastest) x dim1 x dim2; idx is the flat element index.  Returns 0 on an unknown
 * code after filling with the code itself (the reference's final else-branch).
 * ------------------------------------------------------------------------------------------- */
ORC_API int orc_init_pattern(float code, uint32_t dim0, uint32_t dim1, uint32_t dim2, float* out)
{
    int known = 1;
    for (uint32_t bt = 0; bt < dim2; ++bt)
        for (uint32_t ch = 0; ch < dim1; ++ch)
            for (uint32_t i = 0; i < dim0; ++i) {
                uint32_t idx = dim0 * (dim1 * bt + ch) + i;
                float v;
                if (code == 0.0f) v = 0.0f;          /* init_type 0: buffer left as allocated */
                else if (code == 0.5f) v = 0.0f;
                else if (code == 1.0f) v = 1.0f;
                else if (code == 2.0f) v = 1.0f * (float)idx;
                else if (code == 2.1f) v = 0.01f * (float)(idx % 1137u);
                else if (code == 2.2f) v = (float)(i + 1) * 0.01f + (float)ch * 1.0f + (float)bt * 100.0f;
                else if (code == 2.3f) v = 0.1f * (float)(idx % 17u);
                else if (code == 2.4f) v = 1.0f * (float)(idx % 7u);
                else if (code == -1.0f) v = -1.0f;
                else if (code == -2.0f) v = -1.0f * (float)idx;
                else if (code == -2.1f) v = -0.01f * (float)(idx % 1137u);
                else if (code == -2.2f) v = (float)(i + 1) * -0.01f + (float)ch * -1.0f + (float)bt * -100.0f;
                else if (code == -2.3f) v = -0.1f * (float)(idx % 17u);
                else if (code == -2.4f) v = -1.0f * (float)(idx % 11u);
                else { v = code; known = 0; }
                out[idx] = v;
            }
    return known;
}

/* ---------------------------------------------------------------------------------------------
 * GEMM oracles.  Column-major BLAS convention, elements in float:
 *   op(A)(m,k) = trans_a ? A[k + m*lda] : A[m + k*lda]
 *   op(B)(k,n) = trans_b ? B[n + k*ldb] : B[k + n*ldb]
 *   D(m,n)     = alpha * sum_k op(A)(m,k) op(B)(k,n) + beta * C(m,n),  C/D at [m + n*ld]
 * Batch b offsets every operand by b * stride_x.  C may be NULL when beta == 0.
 * Columns [n_begin, n_end) only are computed (the CPU baseline times a subset of columns).
 * ------------------------------------------------------------------------------------------- */
typedef struct {
    int trans_a, trans_b;
    int64_t M, N, K, batch;
    float alpha, beta;
    const float *A, *B, *C;
    int64_t lda, ldb, ldc, ldd, sa, sb, sc, sd;
    float* D;
    double* D64;
    int64_t n_begin, n_end;
    /* packed K-contiguous copies: Ap[b][m][k], Bp[b][n][k] (the reference's TN storage) */
    float *Ap, *Bp;
} orc_job;

static void pack_operands(orc_job* j)
{
    const int64_t M = j->M, N = j->N, K = j->K;
    for (int64_t b = 0; b < j->batch; ++b) {
        const float* A = j->A + b * j->sa;
        const float* B = j->B + b * j->sb;
        float* Ap = j->Ap + b * M * K;
        float* Bp = j->Bp + b * N * K;
        for (int64_t m = 0; m < M; ++m)
            for (int64_t k = 0; k < K; ++k)
                Ap[m * K + k] = j->trans_a ? A[k + m * j->lda] : A[m + k * j->lda];
        for (int64_t n = 0; n < N; ++n)
            for (int64_t k = 0; k < K; ++k)
                Bp[n * K + k] = j->trans_b ? B[n + k * j->ldb] : B[k + n * j->ldb];
    }
}

/* The reference loop (src/gemmMfma.cpp:325-345) over the packed TN storage. */
static void* run_f32(void* arg)
{
    orc_job* j = (orc_job*)arg;
    const int64_t M = j->M, K = j->K, N = j->N;
    for (int64_t b = 0; b < j->batch; ++b)
        for (int64_t n = j->n_begin; n < j->n_end; ++n)
            for (int64_t m = 0; m < M; ++m) {
                const float* a = j->Ap + b * M * K + m * K;
                const float* bb = j->Bp + b * N * K + n * K;
                float t_sum = 0.0f;
                for (int64_t k = 0; k < K; ++k)
                    t_sum += a[k] * bb[k];
                float c = (j->C && j->beta != 0.0f) ? j->C[b * j->sc + m + n * j->ldc] : 0.0f;
                t_sum = j->alpha * t_sum + j->beta * c;
                j->D[b * j->sd + m + n * j->ldd] = t_sum;
            }
    return NULL;
}

static void* run_f64(void* arg)
{
    orc_job* j = (orc_job*)arg;
    const int64_t M = j->M, K = j->K, N = j->N;
    for (int64_t b = 0; b < j->batch; ++b)
        for (int64_t n = j->n_begin; n < j->n_end; ++n)
            for (int64_t m = 0; m < M; ++m) {
                const float* a = j->Ap + b * M * K + m * K;
                const float* bb = j->Bp + b * N * K + n * K;
                double t = 0.0;
                for (int64_t k = 0; k < K; ++k) t += (double)a[k] * (double)bb[k];
                double c = (j->C && j->beta != 0.0f) ? (double)j->C[b * j->sc + m + n * j->ldc] : 0.0;
                j->D64[b * j->sd + m + n * j->ldd] = (double)j->alpha * t + (double)j->beta * c;
            }
    return NULL;
}

static int run_threads(orc_job* base, void* (*fn)(void*), int threads)
{
    if (threads < 1) threads = 1;
    int64_t cols = base->n_end - base->n_begin;
    if (cols <= 0) return 0;
    if (threads > cols) threads = (int)cols;
    if (threads == 1) { fn(base); return 0; }
    pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    orc_job* jobs = (orc_job*)malloc(sizeof(orc_job) * (size_t)threads);
    if (!tid || !jobs) { free(tid); free(jobs); return -1; }
    int64_t per = (cols + threads - 1) / threads;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        jobs[t] = *base;
        jobs[t].n_begin = base->n_begin + (int64_t)t * per;
        jobs[t].n_end = jobs[t].n_begin + per;
        if (jobs[t].n_end > base->n_end) jobs[t].n_end = base->n_end;
        if (jobs[t].n_begin >= jobs[t].n_end) break;
        if (pthread_create(&tid[t], NULL, fn, &jobs[t]) != 0) { fn(&jobs[t]); continue; }
        started = t + 1;
    }
    for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
    free(tid);
    free(jobs);
    return 0;
}

static int setup_job(orc_job* j, int trans_a, int trans_b, int64_t M, int64_t N, int64_t K, int64_t batch,
                     float alpha, const float* A, int64_t lda, int64_t sa, const float* B, int64_t ldb,
                     int64_t sb, float beta, const float* C, int64_t ldc, int64_t sc, int64_t ldd, int64_t sd,
                     int64_t n_begin, int64_t n_end)
{
    memset(j, 0, sizeof(*j));
    j->trans_a = trans_a; j->trans_b = trans_b;
    j->M = M; j->N = N; j->K = K; j->batch = batch;
    j->alpha = alpha; j->beta = beta;
    j->A = A; j->B = B; j->C = C;
    j->lda = lda; j->ldb = ldb; j->ldc = ldc; j->ldd = ldd;
    j->sa = sa; j->sb = sb; j->sc = sc; j->sd = sd;
    j->n_begin = n_begin < 0 ? 0 : n_begin;
    j->n_end = (n_end < 0 || n_end > N) ? N : n_end;
    size_t asz = (size_t)(batch * M * K), bsz = (size_t)(batch * N * K);
    j->Ap = (float*)malloc(sizeof(float) * (asz ? asz : 1));
    j->Bp = (float*)malloc(sizeof(float) * (bsz ? bsz : 1));
    if (!j->Ap || !j->Bp) { free(j->Ap); free(j->Bp); return -1; }
    pack_operands(j);
    return 0;
}

/* Reference-parity fp32 loop.  threads > 1 splits the column range (same per-element result). */
ORC_API int orc_gemm_ref_f32(int trans_a, int trans_b, int64_t M, int64_t N, int64_t K, int64_t batch,
                             float alpha, const float* A, int64_t lda, int64_t stride_a,
                             const float* B, int64_t ldb, int64_t stride_b, float beta,
                             const float* C, int64_t ldc, int64_t stride_c,
                             float* D, int64_t ldd, int64_t stride_d,
                             int64_t n_begin, int64_t n_end, int threads)
{
    orc_job j;
    if (setup_job(&j, trans_a, trans_b, M, N, K, batch, alpha, A, lda, stride_a, B, ldb, stride_b, beta, C,
                  ldc, stride_c, ldd, stride_d, n_begin, n_end))
        return -1;
    j.D = D;
    int rc = run_threads(&j, run_f32, threads);
    free(j.Ap); free(j.Bp);
    return rc;
}

/* Same loop accumulated in double: the FP64 host oracle. */
ORC_API int orc_gemm_f64(int trans_a, int trans_b, int64_t M, int64_t N, int64_t K, int64_t batch,
                         float alpha, const float* A, int64_t lda, int64_t stride_a,
                         const float* B, int64_t ldb, int64_t stride_b, float beta,
                         const float* C, int64_t ldc, int64_t stride_c,
                         double* D, int64_t ldd, int64_t stride_d,
                         int64_t n_begin, int64_t n_end, int threads)
{
    orc_job j;
    if (setup_job(&j, trans_a, trans_b, M, N, K, batch, alpha, A, lda, stride_a, B, ldb, stride_b, beta, C,
                  ldc, stride_c, ldd, stride_d, n_begin, n_end))
        return -1;
    j.D64 = D;
    int rc = run_threads(&j, run_f64, threads);
    free(j.Ap); free(j.Bp);
    return rc;
}

/* Timed form of the reference loop for the CPU baseline: runs the loop on already-packed TN storage
 * (Ap: M x K rows, Bp: N x K rows, single batch) over columns [n_begin, n_end), with the reference's
 * alpha*sum + beta*C step (C column-major, ldc; NULL when beta == 0).  Packing is not part of the
 * reference's cpuCompute, so it stays outside the timed call. */
ORC_API int orc_gemm_ref_f32_packed(int64_t M, int64_t N, int64_t K, float alpha, const float* Ap,
                                    const float* Bp, float beta, const float* C, int64_t ldc, float* D,
                                    int64_t ldd, int64_t n_begin, int64_t n_end, int threads)
{
    orc_job j;
    memset(&j, 0, sizeof(j));
    j.M = M; j.N = N; j.K = K; j.batch = 1; j.alpha = alpha; j.beta = C ? beta : 0.0f;
    j.C = C; j.ldc = ldc;
    j.Ap = (float*)Ap; j.Bp = (float*)Bp; j.D = D; j.ldd = ldd;
    j.n_begin = n_begin; j.n_end = n_end > N ? N : n_end;
    return run_threads(&j, run_f32, threads);
}
