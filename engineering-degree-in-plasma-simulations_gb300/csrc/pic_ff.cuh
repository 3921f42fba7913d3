// Double-FP32 ("float-float") arithmetic: a value is hi + lo with |lo| <= ulp(hi) / 2, about 48
// significant bits carried on the FP32 pipe.  The potential is stored this way because FP64 runs
// at a small fraction of the FP32 rate on this GPU.  Error-free transformations used:
//   TwoSum   s + e = a + b exactly                    (Knuth, The Art of Computer Programming, vol. 2)
//   TwoProd  p + e = a * b exactly, e = fma(a, b, -p)   (the FMA form of Dekker's product)
// The code must not be compiled with reassociating (fast-math) options.
#pragma once
#include <cuda_runtime.h>

namespace pic {

struct FF {
    float hi, lo;
};

__host__ __device__ inline FF ff_from_double(double x) {
    float h = (float)x;
    return FF{h, (float)(x - (double)h)};
}
__host__ __device__ inline double ff_to_double(float2 v) { return (double)v.x + (double)v.y; }
__host__ __device__ inline float2 ff_pack(double x) {
    FF f = ff_from_double(x);
    return make_float2(f.hi, f.lo);
}

__device__ __forceinline__ FF two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return FF{s, e};
}
__device__ __forceinline__ FF two_prod(float a, float b) {
    float p = a * b;
    return FF{p, fmaf(a, b, -p)};
}
// renormalised sum of two float-float values
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    FF s = two_sum(a.hi, b.hi);
    return two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ FF ff_add_f(FF a, float b) {
    FF s = two_sum(a.hi, b);
    return two_sum(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }
// a - b for stored values, unnormalised (the high parts exactly, the low parts in FP32)
__device__ __forceinline__ FF ff_diff(float2 a, float2 b) {
    FF d = two_sum(a.x, -b.x);
    d.lo += a.y - b.y;
    return d;
}
// c * x for a float-float constant c and an unnormalised float-float x
__device__ __forceinline__ FF ff_mul(FF c, FF x) {
    FF p = two_prod(c.hi, x.hi);
    p.lo += c.hi * x.lo + c.lo * x.hi;
    return p;
}

}  // namespace pic
