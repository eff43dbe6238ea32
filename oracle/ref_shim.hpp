// OpenCL-C compatibility shim used to compile the reference's kernel sources as host C++
// (oracle/build_ref.py). ORACLE / TEST INFRASTRUCTURE ONLY: the result goes to oracle/_ref/
// and is used to pin the C restatement in oracle/nfx_oracle.c and to make golden vectors.
//
// It supplies what an OpenCL CPU runtime would: vector types with their operators, the
// geometric built-ins, get_global_id, the 64-bit atom_cmpxchg, and the KernelBuilder defines
// (nofluidx3d/KernelBuilder.py:38-52) as run-time globals so one build serves every mesh.
// Work-items run one after another in index order.
#pragma once
#include <cmath>
#include <cstdint>

typedef unsigned int uint;
typedef unsigned long ulong;

#define kernel extern "C"
#define global

template <class S>
struct vec3_t {
    typedef S scalar;
    S x, y, z;
};
typedef vec3_t<double> double3;
typedef vec3_t<float> float3;

template <class V>
inline V mk3(typename V::scalar a, typename V::scalar b, typename V::scalar c) {
    V r;
    r.x = a;
    r.y = b;
    r.z = c;
    return r;
}

#define VOPS(S)                                                                                \
    inline vec3_t<S> operator+(vec3_t<S> a, vec3_t<S> b) { return mk3<vec3_t<S>>(a.x + b.x, a.y + b.y, a.z + b.z); } \
    inline vec3_t<S> operator-(vec3_t<S> a, vec3_t<S> b) { return mk3<vec3_t<S>>(a.x - b.x, a.y - b.y, a.z - b.z); } \
    inline vec3_t<S> operator-(vec3_t<S> a) { return mk3<vec3_t<S>>(-a.x, -a.y, -a.z); }                          \
    inline vec3_t<S> operator*(vec3_t<S> a, S s) { return mk3<vec3_t<S>>(a.x * s, a.y * s, a.z * s); }             \
    inline vec3_t<S> operator*(S s, vec3_t<S> a) { return mk3<vec3_t<S>>(s * a.x, s * a.y, s * a.z); }             \
    inline vec3_t<S> operator/(vec3_t<S> a, S s) { return mk3<vec3_t<S>>(a.x / s, a.y / s, a.z / s); }             \
    inline vec3_t<S>& operator*=(vec3_t<S>& a, S s) { a.x *= s; a.y *= s; a.z *= s; return a; }                   \
    inline S dot(vec3_t<S> a, vec3_t<S> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }                          \
    inline vec3_t<S> cross(vec3_t<S> a, vec3_t<S> b) {                                                            \
        return mk3<vec3_t<S>>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);                \
    }                                                                                                              \
    inline S length(vec3_t<S> a) { return std::sqrt(dot(a, a)); }                                                \
    inline vec3_t<S> normalize(vec3_t<S> a) { return a / length(a); }
VOPS(double)
VOPS(float)
#undef VOPS
// int scalars used with double vectors in the kernels (e.g. `n1 *= -1`)
inline double3& operator*=(double3& a, int s) { return a *= (double)s; }
inline double max(double a, double b) { return std::fmax(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
using std::pow;
using std::sqrt;

// 64-bit compare-and-swap of OpenCL 1.x (work-items are serial here)
inline ulong atom_cmpxchg(volatile ulong* p, ulong cmp, ulong val) {
    ulong old = *p;
    if (old == cmp) *p = val;
    return old;
}

// get_global_id(0) of the work-item being executed
static long g_gid = 0;
inline long get_global_id(int) { return g_gid; }

// KernelBuilder defines, as globals
static long g_np = 0, g_nt = 0;
static double g_E = 0, g_nu = 0, g_mr = 1;
static bool g_svkk = false, g_svk = false, g_mr_model = true;
static double g_force_const = 0.1;
static double g_vv_xi = 0.005;
static bool g_fixed_top_bottom = false;
#define def_pointCount g_np
#define def_tetraCount g_nt
#define INSERT_NUM_POINTS g_np
#define INSERT_NUM_TETRAS g_nt
#define def_tetraYoungsModulus g_E
#define def_tetraPoissonRatio g_nu
#define def_tetraMooneyRivlinRatio g_mr
#define TETRA_SAINT_VENANT_KIRCHHOFF_KELLNBERGER g_svkk
#define TETRA_SAINT_VENANT_KIRCHHOFF g_svk
#define TETRA_MOONEY_RIVLIN g_mr_model
#define def_FORCE_CONST g_force_const
