// Double-word ("float-float") arithmetic for the Krylov solve of UFE_PREC_FP32_PAIR.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2: about 48
// significant bits, against FP64's 53.  Every operation below runs on the FP32 pipe, which on
// GB300 issues many times more operations per clock than the FP64 pipe; the BiCGStab recurrence
// keeps FP64-like rounding behaviour (relative error per operation a few units of 2^-48).
//
// Building blocks, restated from the published algorithms (no library code):
//   TwoSum      Knuth, TAOCP vol. 2, 4.2.2 Theorem B: s = fl(a+b), e = a+b-s exactly.
//   Fast2Sum    Dekker (1971), for |a| >= |b| (or a = 0).
//   TwoProd     with a fused multiply-add: p = fl(a*b), e = fma(a, b, -p) = a*b-p exactly.
//   DW + DW     Joldes, Muller & Popescu, "Tight and rigorous error bounds for basic building
//               blocks of double-word arithmetic", ACM TOMS 44(2), 2017: AccurateDWPlusDW.
//   DW * DW     same paper, DWTimesDW with FMA (error below 5u^2).
//   dot         Ogita, Rump & Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6),
//               2005: Dot2 (TwoProd terms, TwoSum accumulation, one FP32 correction sum), with
//               the hi*lo cross terms of double-word operands added to the correction.
//
// The explicit __fadd_rn/__fmul_rn/__fmaf_rn intrinsics keep the compiler from contracting or
// reordering the error-free transformations.
#pragma once

#include <cuda_runtime.h>

namespace dword {

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

}  // namespace dword

// A double-word scalar.
struct dw {
  float hi, lo;
  __device__ __forceinline__ dw() {}
  __device__ __forceinline__ dw(float h, float l) : hi(h), lo(l) {}
  // nearest double-word to an FP64 value: d - hi is exact in FP64, so only lo rounds
  __device__ __forceinline__ explicit dw(double d) {
    hi = __double2float_rn(d);
    lo = __double2float_rn(d - (double)hi);
  }
  __device__ __forceinline__ double to_double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dw dw_add(dw x, dw y) {
  float sh, sl, th, tl, vh, vl;
  dword::two_sum(x.hi, y.hi, sh, sl);
  dword::two_sum(x.lo, y.lo, th, tl);
  const float c = __fadd_rn(sl, th);
  dword::fast_two_sum(sh, c, vh, vl);
  const float w = __fadd_rn(tl, vl);
  dw z;
  dword::fast_two_sum(vh, w, z.hi, z.lo);
  return z;
}

__device__ __forceinline__ dw dw_neg(dw x) { return dw(-x.hi, -x.lo); }

__device__ __forceinline__ dw dw_mul(dw x, dw y) {
  float ch, cl1;
  dword::two_prod(x.hi, y.hi, ch, cl1);
  const float tl0 = __fmul_rn(x.lo, y.lo);
  const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  const float cl3 = __fadd_rn(cl1, cl2);
  dw z;
  dword::fast_two_sum(ch, cl3, z.hi, z.lo);
  return z;
}

// Dot2 accumulator: the running sum s and one FP32 correction c.
struct dw_acc {
  float s = 0.f, c = 0.f;
  // += (ah + al) * (xh + xl)
  __device__ __forceinline__ void mac(float ah, float al, float xh, float xl) {
    float p, e, t;
    dword::two_prod(ah, xh, p, e);
    dword::two_sum(s, p, s, t);
    c = __fadd_rn(c, __fadd_rn(t, __fmaf_rn(ah, xl, __fmaf_rn(al, xh, e))));
  }
  __device__ __forceinline__ dw result() const {
    dw z;
    dword::two_sum(s, c, z.hi, z.lo);
    return z;
  }
};

// The (u, v) pair of one triangle: hi parts in .x/.y, lo parts in .z/.w (one 16-byte load).
struct __align__(16) dw2 {
  float4 q;
};
// A 2x2 block (uu, uv, vu, vv): hi parts and lo parts.
struct __align__(16) dwblk {
  float4 hi, lo;
};

__device__ __forceinline__ dw dw_u(dw2 a) { return dw(a.q.x, a.q.z); }
__device__ __forceinline__ dw dw_v(dw2 a) { return dw(a.q.y, a.q.w); }
__device__ __forceinline__ dw2 make_dw2(dw u, dw v) { return dw2{make_float4(u.hi, v.hi, u.lo, v.lo)}; }
__device__ __forceinline__ dw2 to_dw2(double2 a) { return make_dw2(dw(a.x), dw(a.y)); }
__device__ __forceinline__ double2 to_double2(dw2 a) { return make_double2(dw_u(a).to_double(), dw_v(a).to_double()); }
__device__ __forceinline__ dwblk to_dwblk(double4 a) {
  const dw x(a.x), y(a.y), z(a.z), w(a.w);
  return dwblk{make_float4(x.hi, y.hi, z.hi, w.hi), make_float4(x.lo, y.lo, z.lo, w.lo)};
}

// Vector operations of the BiCGStab recurrence (the double-word forms of the FP64 ones).
// p_new = r - bw*v + beta*p
__device__ __forceinline__ dw2 v_pupd(dw2 r, dw bw, dw2 v, dw beta, dw2 p) {
  return make_dw2(dw_add(dw_add(dw_u(r), dw_neg(dw_mul(bw, dw_u(v)))), dw_mul(beta, dw_u(p))),
                  dw_add(dw_add(dw_v(r), dw_neg(dw_mul(bw, dw_v(v)))), dw_mul(beta, dw_v(p))));
}
// r - a*v
__device__ __forceinline__ dw2 v_sub_scaled(dw2 r, dw a, dw2 v) {
  return make_dw2(dw_add(dw_u(r), dw_neg(dw_mul(a, dw_u(v)))), dw_add(dw_v(r), dw_neg(dw_mul(a, dw_v(v)))));
}
// x + a*p + w*s
__device__ __forceinline__ dw2 v_xupd(dw2 x, dw a, dw2 p, dw w, dw2 s) {
  return make_dw2(dw_add(dw_add(dw_u(x), dw_mul(a, dw_u(p))), dw_mul(w, dw_u(s))),
                  dw_add(dw_add(dw_v(x), dw_mul(a, dw_v(p))), dw_mul(w, dw_v(s))));
}
// elementwise product (the Jacobi scaling)
__device__ __forceinline__ dw2 v_mul(dw2 d, dw2 y) {
  return make_dw2(dw_mul(dw_u(d), dw_u(y)), dw_mul(dw_v(d), dw_v(y)));
}
// u_a u_b + v_a v_b, returned in FP64 for the grid reductions
__device__ __forceinline__ double v_dot(dw2 a, dw2 b) {
  dw_acc acc;
  acc.mac(a.q.x, a.q.z, b.q.x, b.q.z);
  acc.mac(a.q.y, a.q.w, b.q.y, b.q.w);
  return acc.result().to_double();
}
