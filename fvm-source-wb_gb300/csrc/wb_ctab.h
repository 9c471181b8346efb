// wb_ctab.h -- compile-time Gauss-Legendre / scaled-Legendre tables (generated by
// gen_ctab.py; exact values rounded to double).  The stage kernels use these so that
// the structural zeros and ones of the basis (phi_0 = 1, phi_1(0) = 0, ...) fold away
// once the quadrature loops are unrolled.
#pragma once

namespace wb {

template <int K>
struct CTab;

template <>
struct CTab<0> {
  static __host__ __device__ __forceinline__ constexpr double xq(int q) { return 0.0; }
  static __host__ __device__ __forceinline__ constexpr double wq(int q) { return 2.0; }
  static __host__ __device__ __forceinline__ constexpr double B(int a, int q) { return 1.0; }
  static __host__ __device__ __forceinline__ constexpr double D(int a, int q) { return 0.0; }
  static __host__ __device__ __forceinline__ constexpr double BW(int a, int q) { return 2.0; }
  static __host__ __device__ __forceinline__ constexpr double DW(int a, int q) { return 0.0; }
  static __host__ __device__ __forceinline__ constexpr double Ep(int a) { return 1.0; }
  static __host__ __device__ __forceinline__ constexpr double Em(int a) { return 1.0; }
  static constexpr int NG = 1;
  static __host__ __device__ __forceinline__ constexpr double xg(int g) { return 0.0; }
  static __host__ __device__ __forceinline__ constexpr double Gl(int a, int g) { return 1.0; }
};

template <>
struct CTab<1> {
  static __host__ __device__ __forceinline__ constexpr double xq(int q) { return (q == 0 ? -0.5773502691896257 : 0.5773502691896257); }
  static __host__ __device__ __forceinline__ constexpr double wq(int q) { return (q == 0 ? 1.0 : 1.0); }
  static __host__ __device__ __forceinline__ constexpr double B(int a, int q) { return (a == 0 ? (q == 0 ? 1.0 : 1.0) : (q == 0 ? -1.0 : 1.0)); }
  static __host__ __device__ __forceinline__ constexpr double D(int a, int q) { return (a == 0 ? (q == 0 ? 0.0 : 0.0) : (q == 0 ? 1.7320508075688772 : 1.7320508075688772)); }
  static __host__ __device__ __forceinline__ constexpr double BW(int a, int q) { return (a == 0 ? (q == 0 ? 1.0 : 1.0) : (q == 0 ? -1.0 : 1.0)); }
  static __host__ __device__ __forceinline__ constexpr double DW(int a, int q) { return (a == 0 ? (q == 0 ? 0.0 : 0.0) : (q == 0 ? 1.7320508075688772 : 1.7320508075688772)); }
  static __host__ __device__ __forceinline__ constexpr double Ep(int a) { return (a == 0 ? 1.0 : 1.7320508075688772); }
  static __host__ __device__ __forceinline__ constexpr double Em(int a) { return (a == 0 ? 1.0 : -1.7320508075688772); }
  static constexpr int NG = 2;
  static __host__ __device__ __forceinline__ constexpr double xg(int g) { return (g == 0 ? -1.0 : 1.0); }
  static __host__ __device__ __forceinline__ constexpr double Gl(int a, int g) { return (a == 0 ? (g == 0 ? 1.0 : 1.0) : (g == 0 ? -1.7320508075688772 : 1.7320508075688772)); }
};

template <>
struct CTab<2> {
  static __host__ __device__ __forceinline__ constexpr double xq(int q) { return (q == 0 ? -0.7745966692414834 : (q == 1 ? 0.0 : 0.7745966692414834)); }
  static __host__ __device__ __forceinline__ constexpr double wq(int q) { return (q == 0 ? 0.5555555555555556 : (q == 1 ? 0.8888888888888888 : 0.5555555555555556)); }
  static __host__ __device__ __forceinline__ constexpr double B(int a, int q) { return (a == 0 ? (q == 0 ? 1.0 : (q == 1 ? 1.0 : 1.0)) : (a == 1 ? (q == 0 ? -1.3416407864998738 : (q == 1 ? 0.0 : 1.3416407864998738)) : (q == 0 ? 0.8944271909999159 : (q == 1 ? -1.118033988749895 : 0.8944271909999159)))); }
  static __host__ __device__ __forceinline__ constexpr double D(int a, int q) { return (a == 0 ? (q == 0 ? 0.0 : (q == 1 ? 0.0 : 0.0)) : (a == 1 ? (q == 0 ? 1.7320508075688772 : (q == 1 ? 1.7320508075688772 : 1.7320508075688772)) : (q == 0 ? -5.196152422706632 : (q == 1 ? 0.0 : 5.196152422706632)))); }
  static __host__ __device__ __forceinline__ constexpr double BW(int a, int q) { return (a == 0 ? (q == 0 ? 0.5555555555555556 : (q == 1 ? 0.8888888888888888 : 0.5555555555555556)) : (a == 1 ? (q == 0 ? -0.7453559924999299 : (q == 1 ? 0.0 : 0.7453559924999299)) : (q == 0 ? 0.49690399499995325 : (q == 1 ? -0.9938079899999065 : 0.49690399499995325)))); }
  static __host__ __device__ __forceinline__ constexpr double DW(int a, int q) { return (a == 0 ? (q == 0 ? 0.0 : (q == 1 ? 0.0 : 0.0)) : (a == 1 ? (q == 0 ? 0.9622504486493763 : (q == 1 ? 1.539600717839002 : 0.9622504486493763)) : (q == 0 ? -2.8867513459481287 : (q == 1 ? 0.0 : 2.8867513459481287)))); }
  static __host__ __device__ __forceinline__ constexpr double Ep(int a) { return (a == 0 ? 1.0 : (a == 1 ? 1.7320508075688772 : 2.23606797749979)); }
  static __host__ __device__ __forceinline__ constexpr double Em(int a) { return (a == 0 ? 1.0 : (a == 1 ? -1.7320508075688772 : 2.23606797749979)); }
  static constexpr int NG = 3;
  static __host__ __device__ __forceinline__ constexpr double xg(int g) { return (g == 0 ? -1.0 : (g == 1 ? 0.0 : 1.0)); }
  static __host__ __device__ __forceinline__ constexpr double Gl(int a, int g) { return (a == 0 ? (g == 0 ? 1.0 : (g == 1 ? 1.0 : 1.0)) : (a == 1 ? (g == 0 ? -1.7320508075688772 : (g == 1 ? 0.0 : 1.7320508075688772)) : (g == 0 ? 2.23606797749979 : (g == 1 ? -1.118033988749895 : 2.23606797749979)))); }
};

}  // namespace wb
