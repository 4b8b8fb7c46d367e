// qs_df.cuh -- double-float arithmetic: a value carried as an unevaluated sum
// hi + lo of two floats (about 48 significand bits).  GB300 executes FP64 at a
// small fraction of its FP32 rate, so the bulk FP64-accuracy work of the
// assembled product and of the Krylov vector operations runs here on the FP32
// pipe, with the error-free transformations TwoSum (Knuth) and TwoProd (via
// fma), as in Dekker (1971) and Hida, Li & Bailey's double-double arithmetic.
#pragma once

#include <cuda_runtime.h>

namespace qs {

struct DF {
    float h, l;
};

#ifdef __CUDACC__

__device__ __forceinline__ DF df_two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return DF{s, e};
}

__device__ __forceinline__ DF df_quick(float a, float b) {
    float s = a + b;
    float e = b - (s - a);
    return DF{s, e};
}

// acc += t * x  (t, x double-float)
__device__ __forceinline__ void df_mac(DF& acc, float th, float tl, float xh, float xl) {
    float p = th * xh;
    float pe = fmaf(th, xh, -p);
    pe = fmaf(th, xl, pe);
    pe = fmaf(tl, xh, pe);
    DF s = df_two_sum(acc.h, p);
    acc.h = s.h;
    acc.l = acc.l + (s.l + pe);
}

__device__ __forceinline__ DF df_add(DF a, DF b) {
    DF s = df_two_sum(a.h, b.h);
    s.l += a.l + b.l;
    return df_quick(s.h, s.l);
}

__device__ __forceinline__ DF df_mul(DF a, DF b) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_quick(p, e);
}

__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }

__device__ __forceinline__ double df_to_double(DF a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ DF df_from_double(double v) {
    float h = __double2float_rn(v);
    float l = __double2float_rn(v - (double)h);
    return DF{h, l};
}

__device__ __forceinline__ DF df_shfl_xor(DF a, int o, int w) {
    return DF{__shfl_xor_sync(0xffffffffu, a.h, o, w), __shfl_xor_sync(0xffffffffu, a.l, o, w)};
}

#endif  // __CUDACC__

// host split of a double into hi + lo floats
inline void df_split_host(double v, float& h, float& l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

}  // namespace qs
