// OpenCL C 1.x compatibility layer for running the reference's kernel strings
// on the host CPU (test infrastructure only: the oracle harness, never the product).
//
// The reference keeps all device arithmetic in OpenCL C source strings
// (radon_tgv_primal_dual_3d.py:96-848, radon_tgv_primal_dual_2d.py:95-463).
// translate.py rewrites those strings into C++ that includes this header:
//   (floatN)(a, b, ...)   -> make_vN(a, b, ...)      component-flattening constructor
//   v.s0 / v.x / v.S2     -> v.c[0] / v.c[0] / v.c[2]
//   v.s012                -> v.sw<0,1,2>()           assignable swizzle proxy
// Vector layout follows the OpenCL spec: float3 occupies 16 bytes like float4.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <type_traits>

namespace ocl {

extern thread_local size_t g_gid[3];
extern thread_local size_t g_gsz[3];
static inline size_t get_global_id(int d) { return g_gid[d]; }
static inline size_t get_global_size(int d) { return g_gsz[d]; }

template <int N> struct Vec;

template <int N> struct StorageOf { static constexpr int value = N; };
template <> struct StorageOf<3> { static constexpr int value = 4; };

template <int N, int... I> struct Swz;

template <int N> struct Vec {
  float c[StorageOf<N>::value];
  Vec() { for (auto &x : c) x = 0.f; }
  Vec(float s) { for (int k = 0; k < StorageOf<N>::value; ++k) c[k] = (k < N) ? s : 0.f; }
  template <int... I> Swz<N, I...> sw() { return Swz<N, I...>{this}; }
  template <int... I> Vec<sizeof...(I)> sw() const {
    Vec<sizeof...(I)> r; int k = 0; ((r.c[k++] = c[I]), ...); return r;
  }
};

template <int N, int... I> struct Swz {
  Vec<N> *v;
  static constexpr int M = sizeof...(I);
  operator Vec<M>() const { Vec<M> r; int k = 0; ((r.c[k++] = v->c[I]), ...); return r; }
  Swz &operator=(const Vec<M> &o) { int k = 0; ((v->c[I] = o.c[k++]), ...); return *this; }
  Swz &operator=(float s) { ((v->c[I] = s), ...); return *this; }
  Swz &operator+=(const Vec<M> &o) { int k = 0; ((v->c[I] += o.c[k++]), ...); return *this; }
  Swz &operator-=(const Vec<M> &o) { int k = 0; ((v->c[I] -= o.c[k++]), ...); return *this; }
  Swz &operator/=(float s) { ((v->c[I] /= s), ...); return *this; }
  Swz &operator*=(float s) { ((v->c[I] *= s), ...); return *this; }
};

using float2 = Vec<2>;
using float3 = Vec<3>;
using float4 = Vec<4>;
using float8 = Vec<8>;

}  // namespace ocl

// dims trait for vectors and swizzles (used by make_v)
namespace ocl {
template <class T> struct VDims;
template <int N> struct VDims<Vec<N>> { static constexpr int value = N; };
template <int N, int... I> struct VDims<Swz<N, I...>> { static constexpr int value = sizeof...(I); };

template <int N, class T> inline void put_one(Vec<N> &r, int &k, const T &s) {
  if constexpr (std::is_arithmetic_v<T>) {
    r.c[k++] = (float)s;
  } else {
    constexpr int M = VDims<T>::value;
    Vec<M> t = s;
    for (int j = 0; j < M; ++j) r.c[k++] = t.c[j];
  }
}
template <int N, class... A> inline Vec<N> make_v(const A &...a) {
  Vec<N> r;
  if constexpr (sizeof...(A) == 1 && (std::is_arithmetic_v<A> && ...)) {
    return Vec<N>((float)(a, ...));
  } else {
    int k = 0;
    (put_one<N>(r, k, a), ...);
    return r;
  }
}
template <class... A> inline Vec<2> make_v2(const A &...a) { return make_v<2>(a...); }
template <class... A> inline Vec<3> make_v3(const A &...a) { return make_v<3>(a...); }
template <class... A> inline Vec<4> make_v4(const A &...a) { return make_v<4>(a...); }
template <class... A> inline Vec<8> make_v8(const A &...a) { return make_v<8>(a...); }

// ---- arithmetic (non-template so swizzle proxies convert implicitly) -------
#define OCL_VEC_OPS(N)                                                                   \
  inline Vec<N> operator-(const Vec<N> &a) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = -a.c[k]; return r; } \
  inline Vec<N> operator+(const Vec<N> &a, const Vec<N> &b) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] + b.c[k]; return r; } \
  inline Vec<N> operator-(const Vec<N> &a, const Vec<N> &b) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] - b.c[k]; return r; } \
  inline Vec<N> operator*(const Vec<N> &a, const Vec<N> &b) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] * b.c[k]; return r; } \
  inline Vec<N> operator/(const Vec<N> &a, const Vec<N> &b) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] / b.c[k]; return r; } \
  inline Vec<N> operator*(float s, const Vec<N> &b) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = s * b.c[k]; return r; } \
  inline Vec<N> operator*(const Vec<N> &a, float s) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] * s; return r; } \
  inline Vec<N> operator/(const Vec<N> &a, float s) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] / s; return r; } \
  inline Vec<N> operator+(const Vec<N> &a, float s) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] + s; return r; } \
  inline Vec<N> operator-(const Vec<N> &a, float s) { Vec<N> r; for (int k = 0; k < N; ++k) r.c[k] = a.c[k] - s; return r; } \
  inline Vec<N> &operator+=(Vec<N> &a, const Vec<N> &b) { for (int k = 0; k < N; ++k) a.c[k] += b.c[k]; return a; } \
  inline Vec<N> &operator-=(Vec<N> &a, const Vec<N> &b) { for (int k = 0; k < N; ++k) a.c[k] -= b.c[k]; return a; } \
  inline Vec<N> &operator/=(Vec<N> &a, float s) { for (int k = 0; k < N; ++k) a.c[k] /= s; return a; }
OCL_VEC_OPS(2)
OCL_VEC_OPS(3)
OCL_VEC_OPS(4)
OCL_VEC_OPS(8)
#undef OCL_VEC_OPS

// ---- built-ins (OpenCL C 1.2 semantics) -------------------------------------
inline float hypot(float a, float b) { return ::hypotf(a, b); }
inline float sqrt(float a) { return ::sqrtf(a); }
inline float fabs(float a) { return ::fabsf(a); }
inline float atan(float a) { return ::atanf(a); }
inline float cos(float a) { return ::cosf(a); }
inline float pow(float a, float b) { return ::powf(a, b); }
inline float min(float a, float b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline float fract(float x, float *ip) {
  float fl = ::floorf(x);
  *ip = fl;
  float r = x - fl;
  const float lim = 0x1.fffffep-1f;
  return r < lim ? r : lim;
}
inline float dot(const Vec<4> &a, const Vec<4> &b) {
  return a.c[0] * b.c[0] + a.c[1] * b.c[1] + a.c[2] * b.c[2] + a.c[3] * b.c[3];
}

}  // namespace ocl
