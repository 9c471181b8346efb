// wb_stage_instances.h -- the compiled stage kernels, one line each: precision tag, element
// type, degree K, basis tag and value (q = tensor Q_k = 0, p = total degree P_k = 1; K = 0
// has one mode and is compiled once, as p), tile TX x TY, the variant mask VAR
// (WB_VAR_POSITIVITY = 1: the positivity limiter compiled in; WB_VAR_HLLC = 2: the HLLC
// face flux) and CPT, the cells per thread (the CTA has TX * TY / CPT threads).  Variant 0
// is compiled for every tile shape; the other variants for the default tile of each
// precision (FP32 32x8, FP64 16x8, one cell per thread), which the dispatch then uses.
// The tile shapes of one (precision, degree, basis) are the autotuner's candidates.
// build.py makes one translation unit per line (parallel nvcc), and wb_stage_dispatch.cu
// picks the kernel at launch from the same list.
//
// The batched form's kernels (k_batch_stage, FP32, total-degree basis) are listed in
// WB_BATCH_INSTANCES: degree K, tile TX x TY, positivity limiter POS, cells per thread CPT.
#pragma once

#define WB_STAGE_INSTANCES(X) \
  X(f32, float, 0, p, 1, 32, 8, 0, 1) \
  X(f32, float, 0, p, 1, 16, 16, 0, 1) \
  X(f32, float, 0, p, 1, 32, 16, 0, 2) \
  X(f32, float, 0, p, 1, 32, 32, 0, 4) \
  X(f32, float, 0, p, 1, 32, 8, 2, 1) \
  X(f32, float, 1, q, 0, 32, 8, 0, 1) \
  X(f32, float, 1, q, 0, 16, 16, 0, 1) \
  X(f32, float, 1, q, 0, 32, 8, 1, 1) \
  X(f32, float, 1, q, 0, 32, 8, 2, 1) \
  X(f32, float, 1, q, 0, 32, 8, 3, 1) \
  X(f32, float, 1, p, 1, 32, 8, 0, 1) \
  X(f32, float, 1, p, 1, 16, 16, 0, 1) \
  X(f32, float, 1, p, 1, 32, 16, 0, 2) \
  X(f32, float, 1, p, 1, 32, 8, 1, 1) \
  X(f32, float, 1, p, 1, 32, 8, 2, 1) \
  X(f32, float, 1, p, 1, 32, 8, 3, 1) \
  X(f32, float, 2, q, 0, 32, 8, 0, 1) \
  X(f32, float, 2, q, 0, 16, 16, 0, 1) \
  X(f32, float, 2, q, 0, 32, 8, 1, 1) \
  X(f32, float, 2, q, 0, 32, 8, 2, 1) \
  X(f32, float, 2, q, 0, 32, 8, 3, 1) \
  X(f32, float, 2, p, 1, 32, 8, 0, 1) \
  X(f32, float, 2, p, 1, 16, 16, 0, 1) \
  X(f32, float, 2, p, 1, 32, 16, 0, 2) \
  X(f32, float, 2, p, 1, 32, 8, 1, 1) \
  X(f32, float, 2, p, 1, 32, 8, 2, 1) \
  X(f32, float, 2, p, 1, 32, 8, 3, 1) \
  X(f64, double, 0, p, 1, 16, 8, 0, 1) \
  X(f64, double, 0, p, 1, 16, 4, 0, 1) \
  X(f64, double, 0, p, 1, 16, 8, 2, 1) \
  X(f64, double, 1, q, 0, 16, 8, 0, 1) \
  X(f64, double, 1, q, 0, 16, 4, 0, 1) \
  X(f64, double, 1, q, 0, 16, 8, 1, 1) \
  X(f64, double, 1, q, 0, 16, 8, 2, 1) \
  X(f64, double, 1, q, 0, 16, 8, 3, 1) \
  X(f64, double, 1, p, 1, 16, 8, 0, 1) \
  X(f64, double, 1, p, 1, 16, 4, 0, 1) \
  X(f64, double, 1, p, 1, 16, 8, 1, 1) \
  X(f64, double, 1, p, 1, 16, 8, 2, 1) \
  X(f64, double, 1, p, 1, 16, 8, 3, 1) \
  X(f64, double, 2, q, 0, 16, 8, 0, 1) \
  X(f64, double, 2, q, 0, 16, 4, 0, 1) \
  X(f64, double, 2, q, 0, 16, 8, 1, 1) \
  X(f64, double, 2, q, 0, 16, 8, 2, 1) \
  X(f64, double, 2, q, 0, 16, 8, 3, 1) \
  X(f64, double, 2, p, 1, 16, 8, 0, 1) \
  X(f64, double, 2, p, 1, 16, 4, 0, 1) \
  X(f64, double, 2, p, 1, 16, 8, 1, 1) \
  X(f64, double, 2, p, 1, 16, 8, 2, 1) \
  X(f64, double, 2, p, 1, 16, 8, 3, 1)

#define WB_STAGE_INSTANCE_NAME(P, K, BT, TX, TY, VAR, CPT) \
  launch_stage_##P##_k##K##BT##_##TX##x##TY##_##VAR##_c##CPT

#define WB_BATCH_INSTANCES(X) \
  X(0, 32, 8, 0, 1) \
  X(0, 16, 16, 0, 1) \
  X(0, 32, 16, 0, 2) \
  X(0, 32, 32, 0, 4) \
  X(1, 32, 8, 0, 1) \
  X(1, 16, 16, 0, 1) \
  X(1, 32, 16, 0, 2) \
  X(1, 32, 8, 1, 1) \
  X(1, 16, 16, 1, 1) \
  X(1, 32, 16, 1, 2) \
  X(2, 32, 8, 0, 1) \
  X(2, 16, 16, 0, 1) \
  X(2, 32, 16, 0, 2) \
  X(2, 32, 8, 1, 1) \
  X(2, 16, 16, 1, 1) \
  X(2, 32, 16, 1, 2)

#define WB_BATCH_INSTANCE_NAME(K, TX, TY, POS, CPT) launch_batch_k##K##_##TX##x##TY##_##POS##_c##CPT
