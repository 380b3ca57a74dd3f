// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
// Exposes the reference's own host converters (inc/ff_utils.h:90-127, compiled in place from the
// reference tree by oracle/Makefile target `ref`) under a C ABI, so the restated converters in
// tl_oracle.c can be pinned against the reference itself.  Nothing here is product code.
#include "ff_utils.h"

extern "C" {
__attribute__((visibility("default"))) unsigned short ref_cvt_f32_to_f16(float f)
{ return (unsigned short)feifei::cvtFP32toFP16(f); }
__attribute__((visibility("default"))) float ref_cvt_f16_to_f32(unsigned short h)
{ return feifei::cvtFP16toFP32(h); }
__attribute__((visibility("default"))) unsigned short ref_cvt_f32_to_bf16(float f)
{ return (unsigned short)feifei::cvtFP32toBF16(f); }
__attribute__((visibility("default"))) float ref_cvt_bf16_to_f32(unsigned short b)
{ return feifei::cvtBF16toFP32(b); }
}

// Bulk forms: values travel by pointer so NaN payloads reach the reference code unchanged.
extern "C" {
__attribute__((visibility("default"))) void ref_cvt_f32_to_f16_n(const float* x, unsigned short* y, long n)
{ for (long i = 0; i < n; ++i) y[i] = (unsigned short)feifei::cvtFP32toFP16(x[i]); }
__attribute__((visibility("default"))) void ref_cvt_f16_to_f32_n(const unsigned short* x, float* y, long n)
{ for (long i = 0; i < n; ++i) y[i] = feifei::cvtFP16toFP32(x[i]); }
__attribute__((visibility("default"))) void ref_cvt_f32_to_bf16_n(const float* x, unsigned short* y, long n)
{ for (long i = 0; i < n; ++i) y[i] = (unsigned short)feifei::cvtFP32toBF16(x[i]); }
__attribute__((visibility("default"))) void ref_cvt_bf16_to_f32_n(const unsigned short* x, float* y, long n)
{ for (long i = 0; i < n; ++i) y[i] = feifei::cvtBF16toFP32(x[i]); }
}
