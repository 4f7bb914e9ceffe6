// Double-single accumulation (value = hi + lo, two floats) by error-free
// transformations (Dekker / Knuth): the product a*b = p + e exactly with
// p = fl(a*b), e = fma(a, b, -p); the sum s + p = t + err exactly with TwoSum.
#pragma once

namespace mnpbem {

struct DS { float hi, lo; };

__device__ __forceinline__ void ds_acc_prod(DS& s, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float t = s.hi + p;
  const float bp = t - s.hi;
  const float err = (s.hi - (t - bp)) + (p - bp);
  s.hi = t;
  s.lo += err + e;
}
__device__ __forceinline__ DS ds_add(DS a, DS b) {
  const float t = a.hi + b.hi;
  const float bp = t - a.hi;
  const float err = (a.hi - (t - bp)) + (b.hi - bp);
  const float lo = a.lo + b.lo + err;
  DS r;
  r.hi = t + lo;                 // renormalise (FastTwoSum)
  r.lo = lo - (r.hi - t);
  return r;
}

// complex (ah + al) * (xh + xl) added to (re, im): exact products of the high
// parts, first-order corrections from the low parts (relative size 2^-24)
__device__ __forceinline__ void ds_cfma(DS& re, DS& im, float2 ah, float2 al, float2 xh, float2 xl) {
  ds_acc_prod(re, ah.x, xh.x);
  ds_acc_prod(re, -ah.y, xh.y);
  ds_acc_prod(im, ah.x, xh.y);
  ds_acc_prod(im, ah.y, xh.x);
  re.lo += (ah.x * xl.x - ah.y * xl.y) + (al.x * xh.x - al.y * xh.y);
  im.lo += (ah.x * xl.y + ah.y * xl.x) + (al.x * xh.y + al.y * xh.x);
}

// double <-> (hi, lo) split; a complex128 value as float4 (hi.x, hi.y, lo.x, lo.y)
__device__ __forceinline__ float4 split4(double2 v) {
  const float hx = (float)v.x, hy = (float)v.y;
  return make_float4(hx, hy, (float)(v.x - (double)hx), (float)(v.y - (double)hy));
}
__device__ __forceinline__ double2 join4(float4 v) {
  return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
}

}  // namespace mnpbem
