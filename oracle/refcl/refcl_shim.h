/*
 * refcl_shim.h -- lets the reference's OpenCL C kernels (res/*.cl) compile as
 * host C++ for the CPU oracle "refcl".  TEST INFRASTRUCTURE ONLY.
 *
 * Provides what an OpenCL 1.2 runtime would: vector types with component
 * access and indexing, dot(), min/max (taken with fmin/fmax semantics for
 * floating point: a NaN argument yields the other argument), and the
 * work-item functions, backed by thread-local ids set by the driver.
 * The program-scope `real` is chosen by REFCL_REAL before this is included.
 */
#pragma once
#include <cmath>
#include <cstddef>
#include <cstring>
#include <cfloat>
#include <type_traits>

using std::fabs;
using std::sqrt;

typedef REFCL_REAL real;

struct real4 {
    real x, y, z, w;
    real& operator[](int i) { return (&x)[i]; }
    const real& operator[](int i) const { return (&x)[i]; }
};
struct int4 {
    int x, y, z, w;
    int& operator[](int i) { return (&x)[i]; }
    const int& operator[](int i) const { return (&x)[i]; }
};
struct int2 {
    int x, y;
    int& operator[](int i) { return (&x)[i]; }
};

struct float4 {
    float x, y, z, w;
};

static inline real4 make_real4(real a, real b, real c, real d) { real4 r = {a, b, c, d}; return r; }
static inline float4 make_float4(double a, double b, double c, double d) {
    float4 r = {(float)a, (float)b, (float)c, (float)d};
    return r;
}
static inline int4 make_int4(long a, long b, long c, long d) { int4 r = {(int)a, (int)b, (int)c, (int)d}; return r; }
static inline int2 make_int2(long a, long b) { int2 r = {(int)a, (int)b}; return r; }

static inline real4 operator+(real4 a, real4 b) { return make_real4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline real4 operator-(real4 a, real4 b) { return make_real4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline real4 operator*(real s, real4 v) { return make_real4(s * v.x, s * v.y, s * v.z, s * v.w); }
static inline real4 operator*(real4 v, real s) { return make_real4(v.x * s, v.y * s, v.z * s, v.w * s); }
static inline real4 operator/(real4 v, real s) { return make_real4(v.x / s, v.y / s, v.z / s, v.w / s); }
/* dot product summed x, y, z, w in that order, each product rounded */
static inline real dot(real4 a, real4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }

/* .xy = .yx and .xz = .zx swizzle assignments, rewritten to calls */
static inline void refcl_swap_xy(real4& v) { real t = v.x; v.x = v.y; v.y = t; }
static inline void refcl_swap_xz(real4& v) { real t = v.x; v.x = v.z; v.z = t; }

/* OpenCL min/max on floating types: fmin/fmax, in the promoted type of the arguments */
template <class A, class B>
static inline typename std::common_type<A, B>::type min(A a, B b) {
    typedef typename std::common_type<A, B>::type T;
    if (std::is_floating_point<T>::value) return (T)std::fmin((T)a, (T)b);
    return (T)a < (T)b ? (T)a : (T)b;
}
template <class A, class B>
static inline typename std::common_type<A, B>::type max(A a, B b) {
    typedef typename std::common_type<A, B>::type T;
    if (std::is_floating_point<T>::value) return (T)std::fmax((T)a, (T)b);
    return (T)a > (T)b ? (T)a : (T)b;
}

/* work-item functions: the driver sets these before calling a kernel */
extern thread_local size_t refcl_gid[3];
extern thread_local size_t refcl_gsize[3];
static inline size_t get_global_id(int d) { return d < 3 ? refcl_gid[d] : 0; }
static inline size_t get_global_size(int d) { return d < 3 ? refcl_gsize[d] : 1; }
/* findMinTimestep/dotBuffer use work-group reductions; the driver never calls them
 * (the reduction is done by the driver), so these only need to compile. */
static inline size_t get_local_id(int) { return 0; }
static inline size_t get_local_size(int) { return 1; }
static inline size_t get_group_id(int d) { return get_global_id(d); }
#define CLK_LOCAL_MEM_FENCE 0
static inline void barrier(int) {}
