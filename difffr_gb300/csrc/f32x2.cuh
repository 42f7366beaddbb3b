// f32x2.cuh — packed FP32 pairs: Blackwell's f32x2 arithmetic does two FP32 operations
// per instruction. Used by the learned warm start's activation layers.
//
// A packed operation on its own rounds as its scalar .rn form (measured: mul, add and fma
// on 8M random pairs, no difference). In context the results can still differ from the
// scalar form's in the last bit: a packed product that feeds only a packed sum came out
// fused into one multiply-add (a squared distance (dx^2 + dy^2) + dz^2 differed from the
// IEEE single-precision value in 16 % of 8M cases, while the scalar .rn form matched it in
// all of them). So these are for arithmetic that a tolerance covers, not for exact
// predicates: the neighbour test keeps its scalar .rn form.
#pragma once
#include <cuda_runtime.h>

namespace dfsph {

static __device__ __forceinline__ unsigned long long f2_bits(float2 v) {
  return (unsigned long long)__float_as_uint(v.x) | ((unsigned long long)__float_as_uint(v.y) << 32);
}
static __device__ __forceinline__ float2 f2_of(unsigned long long u) {
  return make_float2(__uint_as_float((unsigned)u), __uint_as_float((unsigned)(u >> 32)));
}
static __device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
  return f2_of(d);
}
static __device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_of(d);
}
static __device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_of(d);
}
}  // namespace dfsph
