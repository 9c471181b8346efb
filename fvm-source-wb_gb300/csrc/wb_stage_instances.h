// wb_stage_instances.h -- the compiled stage kernels, one line each: precision tag, element
// type, degree K, basis tag and value (q = tensor Q_k = 0, p = total degree P_k = 1; K = 0
// has one mode and is compiled once, as p), tile TX x TY, and the variant mask VAR
// (WB_VAR_POSITIVITY = 1: the positivity limiter compiled in; WB_VAR_HLLC = 2: the HLLC
// face flux).  Variant 0 is compiled for every tile shape; the other variants for the
// default tile of each precision (FP32 32x8, FP64 16x8), which the dispatch then uses.
// build.py makes one translation unit per line (parallel nvcc), and wb_stage_dispatch.cu
// picks the kernel at launch from the same list.
#pragma once

#define WB_STAGE_INSTANCES(X) \
  X(f32, float, 0, p, 1, 32, 8, 0) \
  X(f32, float, 0, p, 1, 16, 16, 0) \
  X(f32, float, 0, p, 1, 32, 8, 2) \
  X(f32, float, 1, q, 0, 32, 8, 0) \
  X(f32, float, 1, q, 0, 16, 16, 0) \
  X(f32, float, 1, q, 0, 32, 8, 1) \
  X(f32, float, 1, q, 0, 32, 8, 2) \
  X(f32, float, 1, q, 0, 32, 8, 3) \
  X(f32, float, 1, p, 1, 32, 8, 0) \
  X(f32, float, 1, p, 1, 16, 16, 0) \
  X(f32, float, 1, p, 1, 32, 8, 1) \
  X(f32, float, 1, p, 1, 32, 8, 2) \
  X(f32, float, 1, p, 1, 32, 8, 3) \
  X(f32, float, 2, q, 0, 32, 8, 0) \
  X(f32, float, 2, q, 0, 16, 16, 0) \
  X(f32, float, 2, q, 0, 32, 8, 1) \
  X(f32, float, 2, q, 0, 32, 8, 2) \
  X(f32, float, 2, q, 0, 32, 8, 3) \
  X(f32, float, 2, p, 1, 32, 8, 0) \
  X(f32, float, 2, p, 1, 16, 16, 0) \
  X(f32, float, 2, p, 1, 32, 8, 1) \
  X(f32, float, 2, p, 1, 32, 8, 2) \
  X(f32, float, 2, p, 1, 32, 8, 3) \
  X(f64, double, 0, p, 1, 16, 8, 0) \
  X(f64, double, 0, p, 1, 16, 4, 0) \
  X(f64, double, 0, p, 1, 16, 8, 2) \
  X(f64, double, 1, q, 0, 16, 8, 0) \
  X(f64, double, 1, q, 0, 16, 4, 0) \
  X(f64, double, 1, q, 0, 16, 8, 1) \
  X(f64, double, 1, q, 0, 16, 8, 2) \
  X(f64, double, 1, q, 0, 16, 8, 3) \
  X(f64, double, 1, p, 1, 16, 8, 0) \
  X(f64, double, 1, p, 1, 16, 4, 0) \
  X(f64, double, 1, p, 1, 16, 8, 1) \
  X(f64, double, 1, p, 1, 16, 8, 2) \
  X(f64, double, 1, p, 1, 16, 8, 3) \
  X(f64, double, 2, q, 0, 16, 8, 0) \
  X(f64, double, 2, q, 0, 16, 4, 0) \
  X(f64, double, 2, q, 0, 16, 8, 1) \
  X(f64, double, 2, q, 0, 16, 8, 2) \
  X(f64, double, 2, q, 0, 16, 8, 3) \
  X(f64, double, 2, p, 1, 16, 8, 0) \
  X(f64, double, 2, p, 1, 16, 4, 0) \
  X(f64, double, 2, p, 1, 16, 8, 1) \
  X(f64, double, 2, p, 1, 16, 8, 2) \
  X(f64, double, 2, p, 1, 16, 8, 3)

#define WB_STAGE_INSTANCE_NAME(P, K, BT, TX, TY, VAR) launch_stage_##P##_k##K##BT##_##TX##x##TY##_##VAR
