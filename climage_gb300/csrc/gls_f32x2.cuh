// gls_f32x2.cuh -- packed fp32 pairs (sm_100 family: add/sub/mul/fma.rn.f32x2).
//
// Each lane of a packed operation is rounded exactly as the scalar operation is (IEEE
// binary32, round to nearest even, no flush of subnormals), so two independent scalar
// chains can run as one packed chain without changing a bit.  The packed forms issue one
// instruction for two results at the same lane throughput, which is what the issue-bound
// pixel kernels gain from them.
//
// One rule keeps them exact: a packed product must never be an operand of a packed add or
// subtract.  The assembler of this toolchain (CUDA 13.0) contracts mul.rn.f32x2 followed
// by add.rn.f32x2 into one fma.rn.f32x2 even under --fmad=false (for the __fmul2_rn /
// __fadd2_rn intrinsics, for explicit PTX, and for fma(a, b, -0) as well), which rounds
// once where the scalar code rounds twice.  A product that is summed is therefore formed by
// mul2s (two scalar multiplies, which the assembler keeps separate); mul2 serves only
// products that feed a multiply or the multiplicands of an fma.
#ifndef GLS_F32X2_CUH
#define GLS_F32X2_CUH

#include <cuda_runtime.h>

namespace gls {

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Each operation packs its float operands into 64-bit register pairs inside the PTX
// (mov.b64 {lo, hi}), which the assembler allocates as adjacent registers at no cost.
#define GLS_F32X2_BIN(NAME, OP)                                                                           \
    __device__ __forceinline__ float2 NAME(float2 a, float2 b) {                                          \
        float2 d;                                                                                         \
        asm("{\n.reg .b64 ra, rb, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %5};\n" OP " rd, ra, rb;\n" \
            "mov.b64 {%0, %1}, rd;\n}\n"                                                                   \
            : "=f"(d.x), "=f"(d.y)                                                                        \
            : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                                    \
        return d;                                                                                         \
    }
GLS_F32X2_BIN(add2, "add.rn.f32x2")
GLS_F32X2_BIN(sub2, "sub.rn.f32x2")
// a * b per lane; never add or subtract the result (see above)
GLS_F32X2_BIN(mul2, "mul.rn.f32x2")
#undef GLS_F32X2_BIN

// a * b per lane as two scalar multiplies: safe to add or subtract afterwards
__device__ __forceinline__ float2 mul2s(float2 a, float2 b) {
    return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
// a * b + c per lane, one rounding
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n.reg .b64 ra, rb, rc, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %5};\nmov.b64 rc, {%6, %7};\n"
        "fma.rn.f32x2 rd, ra, rb, rc;\nmov.b64 {%0, %1}, rd;\n}\n"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

// Two float-float accumulators side by side: ff_add / ff_add_prod (gls_device.cuh) per lane.
struct FF2 {
    float2 hi, lo;
};

__device__ __forceinline__ void ff2_zero(FF2& a) {
    a.hi = make_float2(0.0f, 0.0f);
    a.lo = make_float2(0.0f, 0.0f);
}

__device__ __forceinline__ void ff2_add(FF2& a, float2 x) {
    const float2 s = add2(a.hi, x);
    const float2 bb = sub2(s, a.hi);
    const float2 err = add2(sub2(a.hi, sub2(s, bb)), sub2(x, bb));
    a.hi = s;
    a.lo = add2(a.lo, err);
}

__device__ __forceinline__ void ff2_add_prod(FF2& a, float2 x, float2 y) {
    const float2 p = mul2s(x, y);  // summed below: scalar multiplies
    const float2 e = fma2(x, y, make_float2(-p.x, -p.y));
    ff2_add(a, p);
    a.lo = add2(a.lo, e);
}

}  // namespace gls

#endif  // GLS_F32X2_CUH
