// ss_f2.cuh — packed f32x2 arithmetic (sm_100 and later): two FP32 values
// per register pair, each add, multiply and FMA one packed instruction for
// both lanes, rounded to nearest per lane like the scalar forms.  Used by
// the kernels that carry two independent systems per thread (two stream
// particles, two subhalo responses).  Reciprocal and square-root estimates
// stay per lane (the special-function unit has no packed form); their
// Newton refinements are packed.
#pragma once

#include <cuda_runtime.h>

namespace ssg {

using f2 = float2;

__device__ __forceinline__ f2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pr, pa, pb;\n\t"
        "mov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ f2 neg2(f2 a) { return make_float2(-a.x, -a.y); }

// s_rsqrt per lane: estimate, then y - (y/2)(x y^2 - 1) (the same rounded
// values as y + (y/2)(1 - x y^2)).
__device__ __forceinline__ f2 rsqrt2(f2 x) {
    const f2 y = make_float2(rsqrtf(x.x), rsqrtf(x.y));
    const f2 e = fma2(mul2(x, y), y, bc(-1.0f));
    return fma2(mul2(bc(-0.5f), y), e, y);
}

// s_rcp per lane: estimate, then r - r (x r - 1).
__device__ __forceinline__ f2 rcp2(f2 x) {
    const f2 r = make_float2(__fdividef(1.0f, x.x), __fdividef(1.0f, x.y));
    const f2 e = fma2(x, r, bc(-1.0f));
    return fma2(neg2(r), e, r);
}

__device__ __forceinline__ f2 norm2sq(const f2 x[3]) {
    return fma2(x[2], x[2], fma2(x[1], x[1], mul2(x[0], x[0])));
}

}  // namespace ssg
