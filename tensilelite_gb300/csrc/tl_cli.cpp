// tensilelite: command-line GEMM runner over the library's C ABI, taking the reference program's
// options (inc/ff_utils.h:347-361: -d -m -n -k -p -r -s -x -y -z -u -v -l -f -t, long names alike)
// and following its run (src/main.cpp, src/gemmMfma.cpp): buffers padded by -p elements, the
// integer-pattern data with alpha 0.314 and beta 0.2718, one warm-up launch, verification, then -l
// timed launches and a performance summary.
//
// Verification runs the CUDA-core kernel on the same inputs (an independent implementation; the
// integer pattern keeps every partial sum exact, so both must agree) and compares on the host with
// the reference's tolerance of 0.1.  Tile options map to the tensor-core solution: macro tile
// MT0 = z*r*x along m, MT1 = z*s*y along n, -f stages, -u depth; when none is given the heuristic
// picks the tile.  -t 1 drives the Tensile-layout entry (tl_tensile_launch) with a Tensile argument
// buffer, as the reference's -t 1 mode generates the Cijk_Alik_Bljk kernel.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "include/tensilelite.h"

namespace {

struct Opt {
    char s;
    const char* l;
    const char* def;
    const char* help;
};

const Opt kOpts[] = {
    {'d', "data-type", "1", "data type: 1 fp32, 2 fp16, 3 bf16. (1)"},
    {'m', "gemm-m", "1024", "gemm m dim. (1024)"},
    {'n', "gemm-n", "1024", "gemm n dim. (1024)"},
    {'k', "gemm-k", "1024", "gemm k dim. (1024)"},
    {'p', "padding", "64", "elements padding for m/n/k. (64)"},
    {'r', "mfma-pttn0", "1", "mma tiles per wave in m. (1)"},
    {'s', "mfma-pttn1", "1", "mma tiles per wave in n. (1)"},
    {'x', "wave-pttn0", "1", "waves per group in m. (1)"},
    {'y', "wave-pttn1", "1", "waves per group in n. (1)"},
    {'z', "mfma-mn", "32", "mma instruction m/n width. (32)"},
    {'u', "depth-u", "16", "k dim loop unroll. (16)"},
    {'v', "verify", "1", "enable verify. (1)"},
    {'l', "loop", "100", "loop times for perf test. (100)"},
    {'f', "buffer", "3", "shared-memory buffer (stage) number. (3)"},
    {'t', "tensile", "0", "if use tensile format. (0)"},
    {'b', "batch", "1", "batch count. (1)"},
    {'e', "kernel", "auto", "kernel: auto, tcgen05, simt, bf16x3, bf16x6. (auto)"},
};

void help()
{
    printf("usage: tensilelite [options]\n");
    printf("  -h --help          help infomation\n");
    for (const Opt& o : kOpts) printf("  -%c --%-15s %s\n", o.s, o.l, o.help);
}

#define CHECK(call)                                                                                      \
    do {                                                                                                 \
        tl_status st_ = (call);                                                                          \
        if (st_ != TL_SUCCESS) {                                                                         \
            fprintf(stderr, "[ERROR] %s: %s (%s)\n", #call, tl_status_string(st_), tl_last_error_string()); \
            return 2;                                                                                    \
        }                                                                                                \
    } while (0)

float decode(const void* buf, size_t i, int dt)
{
    if (dt == TL_DTYPE_FP32) return static_cast<const float*>(buf)[i];
    const uint16_t b = static_cast<const uint16_t*>(buf)[i];
    if (dt == TL_DTYPE_BF16) {
        uint32_t w = static_cast<uint32_t>(b) << 16;
        float f;
        memcpy(&f, &w, 4);
        return f;
    }
    __half_raw r;
    r.x = b;
    return __half2float(__half(r));
}

}  // namespace

int main(int argc, char* argv[])
{
    setvbuf(stdout, nullptr, _IOLBF, 0);
    std::map<char, std::string> v;
    std::map<char, bool> given;
    for (const Opt& o : kOpts) v[o.s] = o.def;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "-h" || a == "--help") {
            help();
            return 0;
        }
        char key = 0;
        if (a.size() == 2 && a[0] == '-') key = a[1];
        else if (a.rfind("--", 0) == 0)
            for (const Opt& o : kOpts)
                if (a.substr(2) == o.l) key = o.s;
        if (!key || !v.count(key) || i + 1 >= argc) {
            fprintf(stderr, "[ERROR] unknown or incomplete option %s\n", a.c_str());
            help();
            return 1;
        }
        v[key] = argv[++i];
        given[key] = true;
    }
    auto I = [&](char c) { return static_cast<int64_t>(atoll(v[c].c_str())); };
    const int dt = static_cast<int>(I('d'));
    if (dt < 1 || dt > 3) {
        fprintf(stderr, "[ERROR] data type must be 1 (fp32), 2 (fp16) or 3 (bf16)\n");
        return 1;
    }
    const int64_t M = I('m'), N = I('n'), K = I('k'), pad = I('p'), batch = I('b'), loops = I('l');
    const bool verify = I('v') != 0, tensile = I('t') != 0;
    const int esz = dt == TL_DTYPE_FP32 ? 4 : 2;
    const char* dname[] = {"", "FP32", "FP16", "BF16"};

    // the reference's layout: TN column-major, every leading dimension padded (src/gemmMfma.cpp:210-217)
    const int64_t lda = K + pad, ldb = K + pad, ldc = M + pad, ldd = M + pad;
    const int64_t sa = lda * M, sb = ldb * N, sc = ldc * N, sd = ldd * N;
    printf("[INFO] data type = %s\n", dname[dt]);
    printf("[INFO] gemm size: M,N,K,Batch = %lld, %lld, %lld, %lld.\n", (long long)M, (long long)N, (long long)K,
           (long long)batch);
    printf("[INFO] row   stride: A,B,C,D = %lld, %lld, %lld, %lld.\n", (long long)lda, (long long)ldb, (long long)ldc,
           (long long)ldd);
    printf("[INFO] batch stride: A,B,C,D = %lld, %lld, %lld, %lld.\n", (long long)sa, (long long)sb, (long long)sc,
           (long long)sd);
    printf("[INFO] padding = %lld(elements).\n", (long long)pad);

    tl_handle* h = nullptr;
    CHECK(tl_init(&h));
    int sms = 0, ccmaj = 0, ccmin = 0;
    size_t smem = 0;
    CHECK(tl_device_info(h, &sms, &ccmaj, &ccmin, &smem));
    printf("[INFO] device: sm_%d%d, %d SMs, %zu KB shared memory per block.\n", ccmaj, ccmin, sms, smem / 1024);
    void* stream = nullptr;
    CHECK(tl_stream_create(&stream));

    void *A, *B, *C, *D, *R = nullptr;
    CHECK(tl_malloc(&A, static_cast<size_t>(sa * batch) * esz));
    CHECK(tl_malloc(&B, static_cast<size_t>(sb * batch) * esz));
    CHECK(tl_malloc(&C, static_cast<size_t>(sc * batch) * esz));
    CHECK(tl_malloc(&D, static_cast<size_t>(sd * batch) * esz));
    // InitRealData codes of the reference (src/gemmMfma.cpp:231-235)
    CHECK(tl_fill_pattern(static_cast<tl_dtype>(dt), A, sa * batch, 2.4f, stream));
    CHECK(tl_fill_pattern(static_cast<tl_dtype>(dt), B, sb * batch, -2.4f, stream));
    CHECK(tl_fill_pattern(static_cast<tl_dtype>(dt), C, sc * batch, 2.4f, stream));
    CHECK(tl_fill_pattern(static_cast<tl_dtype>(dt), D, sd * batch, 0.5f, stream));
    const float alpha = 0.314f, beta = 0.2718f;

    tl_gemm_problem p;
    CHECK(tl_problem_init(&p, static_cast<tl_dtype>(dt), static_cast<tl_dtype>(dt), TL_OP_T, TL_OP_N, M, N, K));
    p.batch = batch;
    p.lda = lda; p.ldb = ldb; p.ldc = ldc; p.ldd = ldd;
    p.stride_a = sa; p.stride_b = sb; p.stride_c = sc; p.stride_d = sd;
    p.alpha = alpha;
    p.beta = beta;
    if (dt == TL_DTYPE_BF16) p.out_rounding = TL_ROUND_TRUNCATE;   // the reference kernel's bf16 store
    const std::string kname = v['e'];
    p.kernel = kname == "tcgen05" ? TL_KERNEL_TCGEN05 : kname == "simt" ? TL_KERNEL_SIMT
             : kname == "bf16x3"  ? TL_KERNEL_BF16X3 : kname == "bf16x6" ? TL_KERNEL_BF16X6 : TL_KERNEL_AUTO;

    tl_gemm_solution sol;
    const tl_gemm_solution* solp = nullptr;
    const bool tile_given = given['r'] || given['s'] || given['x'] || given['y'] || given['z'] || given['u'] || given['f'];
    if (tile_given && !tensile) {
        CHECK(tl_default_solution(h, &p, &sol));
        if (sol.kernel != TL_KERNEL_SIMT) {
            const int64_t z = I('z');
            sol.macro_tile0 = static_cast<int32_t>(z * I('r') * I('x'));
            sol.macro_tile1 = static_cast<int32_t>(z * I('s') * I('y'));
            if (given['u']) sol.depth_u = static_cast<int32_t>(I('u'));
            if (given['f']) sol.stages = static_cast<int32_t>(I('f'));
        }
        CHECK(tl_check_solution(h, &p, &sol));   // the reference's checkKernelParameters
        solp = &sol;
    } else {
        CHECK(tl_default_solution(h, &p, &sol));
    }
    printf("[INFO] solution: kernel %d, MT = [%d, %d], depth-u %d, stages %d, split-k %d.\n", sol.kernel,
           sol.macro_tile0, sol.macro_tile1, sol.depth_u, sol.stages, sol.split_k);

    // the Tensile-layout argument buffer (src/gemmMfma.cpp:70-103)
    tl_tensile_kernarg ka;
    memset(&ka, 0, sizeof(ka));
    std::string tname;
    if (tensile) {
        ka.size_c = static_cast<uint64_t>(sc * batch);
        ka.size_a = static_cast<uint64_t>(sa * batch);
        ka.size_b = static_cast<uint64_t>(sb * batch);
        ka.d = D; ka.c = C; ka.a = A; ka.b = B;
        if (dt == TL_DTYPE_FP16) {
            ka.alpha_bits = __half_as_ushort(__float2half_rn(alpha));
            ka.beta_bits = __half_as_ushort(__float2half_rn(beta));
        } else {
            memcpy(&ka.alpha_bits, &alpha, 4);
            memcpy(&ka.beta_bits, &beta, 4);
        }
        ka.stride_d0 = static_cast<uint32_t>(ldd); ka.stride_d1 = static_cast<uint32_t>(sd);
        ka.stride_c0 = static_cast<uint32_t>(ldc); ka.stride_c1 = static_cast<uint32_t>(sc);
        ka.stride_a0 = static_cast<uint32_t>(lda); ka.stride_a1 = static_cast<uint32_t>(sa);
        ka.stride_b0 = static_cast<uint32_t>(ldb); ka.stride_b1 = static_cast<uint32_t>(sb);
        ka.sizes_free0 = static_cast<uint32_t>(M); ka.sizes_free1 = static_cast<uint32_t>(N);
        ka.sizes_free2 = static_cast<uint32_t>(batch); ka.sizes_sum0 = static_cast<uint32_t>(K);
        tname = std::string("Cijk_Alik_Bljk_") + (dt == 1 ? "SB" : dt == 2 ? "HBH" : "BBH");
        printf("[INFO] kernel name: %s (Tensile argument layout)\n", tname.c_str());
    }
    auto launch = [&]() -> tl_status {
        if (tensile) return tl_tensile_launch(h, tname.c_str(), &ka, TL_TENSILE_KERNARG_BYTES, stream);
        return tl_gemm(h, &p, solp, D, C, A, B, stream);
    };

    // warm up (D = alpha A^T B + beta C does not read D, so repeated launches give the same D)
    CHECK(launch());
    CHECK(tl_stream_synchronize(stream));
    CHECK(tl_device_status(h, stream));

    if (verify && !tensile) {
        CHECK(tl_malloc(&R, static_cast<size_t>(sd * batch) * esz));
        tl_gemm_problem q = p;
        q.kernel = TL_KERNEL_SIMT;
        CHECK(tl_gemm(h, &q, nullptr, R, C, A, B, stream));
        CHECK(tl_stream_synchronize(stream));
        const size_t bytes = static_cast<size_t>(sd * batch) * esz;
        std::vector<unsigned char> hd(bytes), hr(bytes);
        CHECK(tl_memcpy_d2h(hd.data(), D, bytes, stream));
        CHECK(tl_memcpy_d2h(hr.data(), R, bytes, stream));
        CHECK(tl_stream_synchronize(stream));
        bool pass = true;
        double maxdiff = 0.0;
        for (int64_t b = 0; b < batch && pass; ++b)
            for (int64_t n = 0; n < N && pass; ++n)
                for (int64_t m = 0; m < M; ++m) {
                    const size_t idx = static_cast<size_t>(b * sd + n * ldd + m);
                    const float g = decode(hd.data(), idx, dt), r = decode(hr.data(), idx, dt);
                    const double diff = std::fabs(static_cast<double>(g) - r);
                    if (diff > maxdiff) maxdiff = diff;
                    if (!(diff <= 0.1)) {
                        printf("[WARNING] Verify Failed! [%zu]:gpu=%.2f,ref=%.2f\n", idx, g, r);
                        pass = false;
                        break;
                    }
                }
        if (pass) printf("[INFO] Verify Success. (max |diff| vs the CUDA-core kernel = %g)\n", maxdiff);
    }

    printf("[INFO] Launch kernel for %lld times...\n", (long long)loops);
    tl_timer* t = nullptr;
    CHECK(tl_timer_create(&t));
    CHECK(tl_timer_start(t, stream));
    for (int64_t i = 0; i < loops; ++i) CHECK(launch());
    CHECK(tl_timer_stop(t, stream));
    float ms = 0.f;
    CHECK(tl_timer_elapsed_ms(t, &ms));
    CHECK(tl_device_status(h, stream));
    const double sec = loops > 0 ? ms / 1e3 / loops : 0.0;
    const double flops = 2.0 * M * N * K * batch;
    // nominal dense rates of a GB300: 2.25 PFLOP/s fp16/bf16 tensor; fp32 on the CUDA cores
    const double theory = dt == TL_DTYPE_FP32 ? sms * 128.0 * 2.0 * 2.07e9 : 2.25e15;
    printf("[INFO] Elapsed time = %.3f(us)\n", sec * 1e6);
    printf("[INFO] Calculation = %.2f G\n", flops / 1e9);
    printf("[INFO] Performance = %.2f TFLOPs\n", sec > 0 ? flops / sec / 1e12 : 0.0);
    printf("[INFO] Theory Performance = %.2f TFLOPs\n", theory / 1e12);
    printf("[INFO] Efficiency = %.2f%%\n", sec > 0 ? flops / sec / theory * 100.0 : 0.0);

    tl_timer_destroy(t);
    tl_free(A); tl_free(B); tl_free(C); tl_free(D);
    if (R) tl_free(R);
    tl_stream_destroy(stream);
    tl_destroy(h);
    return 0;
}
