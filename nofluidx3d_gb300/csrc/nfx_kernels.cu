// CUDA kernels of the noFluidX3D tetra-mesh step for sm_103a.
//
// One time step is two kernels:
//   k_tet_pass  — one CTA per tile of tetrahedra: stage the tile's nodes (displacement hi/lo)
//                 in shared memory, evaluate each tetra's material law in registers
//                 (tetra.cl:14-182 or InteractionFiniteStrainViscoplastic.cl:1-220), write the
//                 four corner forces to shared memory, sum them per distinct tile node in the
//                 tile's fixed incidence order, and add each node sum to the force accumulator
//                 as 64-bit fixed point (three integer atomics per tile node). This replaces
//                 the reference's 12 FP64 CAS loops per tetra (atomicAdd.cl:1-11) and makes the
//                 accumulated force independent of the order in which tiles finish.
//   k_node_pass — one thread per node: accumulated element force + substrate/plane/sphere
//                 contacts (Substrate.cl, Plane.cl, Sphere.cl), damped velocity Verlet
//                 (VelocityVerlet.cl:1-36) with the displacement carried as float hi + lo,
//                 zeroing of the accumulator, and on record steps the indenter-force readout of
//                 Simulation.py:146-153 / :198-212 reduced per cell in a fixed order.
// Both kernels read their parameters from a per-cell table in device memory (BatchDev): a single
// simulation is a table of one cell, a batch many, and both run this same code. The kernel
// boundary is the step's only global barrier. Time t comes from device memory (start of the
// captured chunk) plus the launch's offset, so a captured CUDA graph of G steps can be replayed
// for any chunk.
#include <cuda_runtime.h>

#include "nfx_internal.h"
#include "nfx_math.cuh"

namespace nfx {

// Programmatic dependent launch of the node pass. Inside a run of steps the node pass is launched
// with programmatic stream serialisation (NFX_PDL_NODE), so its CTAs can be placed on the SMs
// before the element pass has completed: a node-pass CTA computes its prologue (the cell's
// contact positions from the step clock and the cell table, its block's reference box — data the
// element pass does not write, last written by work that completed before the element pass
// started), then waits in griddepcontrol.wait until the element pass has completed and its
// writes are visible, and only then touches the node state. The element pass itself is launched
// in plain stream order and, with NFX_TET_TRIGGER, allows its dependents to launch as soon as each
// of its CTAs starts (launch_dependents), so that node-pass CTAs take the SMs its last CTAs leave.
// A kernel launched without the attribute passes the wait at once.
#ifndef NFX_PDL_NODE
#define NFX_PDL_NODE 1
#endif
#ifndef NFX_TET_TRIGGER
#define NFX_TET_TRIGGER 1
#endif
// The element pass as a dependent launch of the node pass before it (NFX_PDL_TET): it waits as its
// very first instruction, before any read, so it is correct after any predecessor; what it gains
// is only that its CTAs are resident when the node pass completes. The node pass then releases
// its dependents as each of its CTAs starts.
#ifndef NFX_PDL_TET
#define NFX_PDL_TET 1
#endif
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ double contact_pos(const ContactDev& c, long long t) {
    const long long n = c.meta[1];
    if (n > 0) {
        long long k = t - c.meta[0];
        if (k < 0) k = 0;
        if (k >= n) k = n - 1;
        return c.table[k];
    }
    if (c.kind == CONTACT_SUBSTRATE) return c.p0;
    const double tt = (double)t;
    return tt <= c.tmove ? c.p0 - c.v * tt : c.p0 - c.v * c.tmove;
}

// Raise status bits globally and, in a batch, on the cell they belong to (cstat may be null).
__device__ __forceinline__ void raise_status(const StateDev& s, unsigned* cstat, unsigned bits) {
    atomicOr(s.status, bits);
    if (cstat) atomicOr(cstat, bits);
}
// The status word of tile b's cell (looked up only when a status is raised).
__device__ __forceinline__ unsigned* tile_cell_status(const BatchDev& bd, int b) {
    return bd.cell_status ? bd.cell_status + (bd.tile_cell ? bd.tile_cell[b] : 0) : nullptr;
}

// ------------------------------------------------------------------------------------------
// Element pass: shared pieces
// ------------------------------------------------------------------------------------------

// One tetra: displacement differences from the tile's staged node data, the material law, the
// viscoplastic state update (written back with evict-first stores), the four corner forces
// into the shared corner-force slots k*TILE + j (corner-major, so a warp's stores are
// contiguous and free of bank conflicts). Returns true when the tetra is inverted (det F <= 0).
template <int MODEL, int TILE>
__device__ __forceinline__ bool element_law(int j, long long t, float (&d)[3][3], float4 da, float4 db, float2 dc,
                                            float4 pa, float4 pb, float2 pc, float4* s_cf, const StateDev& s,
                                            const MaterialDev& mat, bool write_fields);
template <int MODEL, int TILE>
__device__ __forceinline__ bool element_eval(int j, long long t, uchar4 lc, float4 da, float4 db, float2 dc,
                                             float4 pa, float4 pb, float2 pc, const float4* s_uh,
                                             const float4* s_ul, float4* s_cf, const StateDev& s,
                                             const MaterialDev& mat, bool write_fields) {
    const int li[4] = {lc.x, lc.y, lc.z, lc.w};
    const float4 u0h = s_uh[li[0]], u0l = s_ul[li[0]];
    float d[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float4 h = s_uh[li[k + 1]], l = s_ul[li[k + 1]];
        d[k][0] = (h.x - u0h.x) + (l.x - u0l.x);
        d[k][1] = (h.y - u0h.y) + (l.y - u0l.y);
        d[k][2] = (h.z - u0h.z) + (l.z - u0l.z);
    }
    return element_law<MODEL, TILE>(j, t, d, da, db, dc, pa, pb, pc, s_cf, s, mat, write_fields);
}
template <int MODEL, int TILE>
__device__ __forceinline__ bool element_law(int j, long long t, float (&d)[3][3], float4 da, float4 db, float2 dc,
                                            float4 pa, float4 pb, float2 pc, float4* s_cf, const StateDev& s,
                                            const MaterialDev& mat, bool write_fields) {
    const float Dmi[9] = {da.x, da.y, da.z, da.w, db.x, db.y, db.z, db.w, dc.x};
    const float V0 = dc.y;
    float f[4][3];
    float jm1;
    if (MODEL == MODEL_MR) {
        jm1 = mr_element(d[0], d[1], d[2], Dmi, V0, mat.mu1, mat.mu2, mat.kappa, f);
    } else if (MODEL == MODEL_SVK) {
        jm1 = svk_element(d[0], d[1], d[2], Dmi, V0, mat.mu, mat.kp, f);
    } else if (MODEL == MODEL_SVKK) {
        jm1 = svkk_element(d[0], d[1], d[2], Dmi, V0, mat.mu, mat.kp, f);
    } else {
        VPParams par;
        par.mu1 = mat.mu1;
        par.mu2 = mat.mu2;
        par.kappa = mat.kappa;
        par.flow_exp = mat.flow_exp;
        par.yield = mat.yield;
        par.flow_rate = mat.flow_rate;
        par.hard_thr = mat.hard_thr;
        par.hard_exp = mat.hard_exp;
        float P[9] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w, pc.x};
        float eps = pc.y;
        float dP[9], rate, vm, pr;
        vp_element(d[0], d[1], d[2], Dmi, V0, par, P, eps, dP, rate, f, vm, pr, jm1);
#pragma unroll
        for (int q = 0; q < 9; q++) P[q] += dP[q];
        eps += rate;
        __stcs(s.vp_a + t, make_float4(P[0], P[1], P[2], P[3]));
        __stcs(s.vp_b + t, make_float4(P[4], P[5], P[6], P[7]));
        __stcs(s.vp_c + t, make_float2(P[8], eps));
        if (write_fields) __stcs(s.fields + t, make_float2(vm, pr));
    }
#pragma unroll
    for (int k = 0; k < 4; k++) s_cf[k * TILE + j] = make_float4(f[k][0], f[k][1], f[k][2], 0.f);
    return !(jm1 > -1.0f);
}

// Fixed-point value round(y) of a float y with |y| < 2^62 — equal to __float2ll_rn(y) bit for
// bit — from two 32-bit conversions (64-bit float/integer conversions run on the FP64 pipe,
// which is narrow on this GPU). |y| = hi 2^32 + r with hi = floor(|y| 2^-32) exact and r exact
// in float (r < 2^32 and a multiple of ulp(|y|)); round-to-nearest-even of r equals that of |y|
// minus hi 2^32, and the rounding is symmetric in the sign.
__device__ __forceinline__ long long fix_round(float y) {
    const float a = fabsf(y);
    const unsigned hi = __float2uint_rz(a * 2.3283064365386963e-10f);  // 2^-32
    const float r = fmaf(-(float)hi, 4294967296.0f, a);                 // exact
    const unsigned long long v = ((unsigned long long)hi << 32) + (unsigned long long)__float2uint_rn(r);
    return y < 0.0f ? -(long long)v : (long long)v;
}

// Float value of a fixed-point accumulator word, w 2^-40 rounded to nearest even — bit for bit
// __ll2float_rn(w) * 2^-40 — built from integer operations alone: normalise |w| with a count
// of leading zeros, keep 24 bits, round on the 40 bits below, and assemble sign, exponent and
// mantissa (the float conversions, 64- and 32-bit alike, run on the narrow FP64 pipe).
__device__ __forceinline__ float fix_to_float(unsigned long long w) {
    const long long sw = (long long)w;
    if (sw == 0) return 0.0f;
    const unsigned sign = sw < 0 ? 0x80000000u : 0u;
    unsigned long long a = sw < 0 ? 0ull - w : w;
    const int lz = __clzll((long long)a);
    a <<= lz;  // leading one at bit 63
    unsigned long long m = a >> 40;  // 24 significant bits
    const unsigned long long rem = a & ((1ull << 40) - 1ull), half = 1ull << 39;
    if (rem > half || (rem == half && (m & 1ull))) m++;
    int e = 63 - lz;  // |w| in [2^e, 2^(e+1))
    if (m == (1ull << 24)) {
        m >>= 1;
        e++;
    }
    const unsigned be = (unsigned)(e - 40 + 127);  // times 2^-40; always a normal float
    return __uint_as_float(sign | (be << 23) | ((unsigned)m & 0x7FFFFFu));
}

// One tile node: sum its corner forces in the tile's fixed incidence order and add the sum to
// the global accumulator as 64-bit fixed point, so the total does not depend on the order in
// which tiles finish. Incidence entries are corner-force slots (corner * TILE + local tet). One
// corner per iteration at the 56-register budget (NFX_FLUSH_UNROLL=4 takes four per iteration,
// in the same order: faster at 64 registers, 5 % slower at 56). Returns false when a component of
// the sum exceeds the mesh's per-tile bound fix_max (nothing is added then), which keeps every
// node's accumulator word within its 64-bit range.
#ifndef NFX_FLUSH_UNROLL
#define NFX_FLUSH_UNROLL 1
#endif
template <int TILE>
__device__ __forceinline__ bool node_flush(uint2 node, const unsigned short* inc, const float4* s_cf,
                                           const StateDev& s, long long np, float fix_max) {
    const unsigned first = node.y >> 16, count = node.y & 0xffffu;
    if (count == 0) return true;
    const unsigned short* e = inc + first;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    unsigned q = 0;
#if NFX_FLUSH_UNROLL == 4
    for (; q + 4 <= count; q += 4) {
        const float4 c0 = s_cf[e[q]], c1 = s_cf[e[q + 1]], c2 = s_cf[e[q + 2]], c3 = s_cf[e[q + 3]];
        fx = (((fx + c0.x) + c1.x) + c2.x) + c3.x;
        fy = (((fy + c0.y) + c1.y) + c2.y) + c3.y;
        fz = (((fz + c0.z) + c1.z) + c2.z) + c3.z;
    }
#endif
    for (; q < count; q++) {
        const float4 c = s_cf[e[q]];
        fx += c.x;
        fy += c.y;
        fz += c.z;
    }
    if (!(fabsf(fx) <= fix_max && fabsf(fy) <= fix_max && fabsf(fz) <= fix_max)) return false;
    atomicAdd(s.facc + node.x, (unsigned long long)fix_round(fx * FORCE_FIX_SCALE));
    atomicAdd(s.facc + np + node.x, (unsigned long long)fix_round(fy * FORCE_FIX_SCALE));
    atomicAdd(s.facc + 2 * np + node.x, (unsigned long long)fix_round(fz * FORCE_FIX_SCALE));
    return true;
}

__device__ __forceinline__ bool clock_bit(const unsigned* mask, int k) { return (mask[k >> 5] >> (k & 31)) & 1u; }

// Sphere centre height, radius and decay rate of an integrated sphere contact for one step.
struct SphereIntegralStep {
    float cy_hi, cy_lo, radius, k;
};

// Integrated sphere contact of one tetra (InteractionSphereIntegral.cl:22-85): the repulsive
// density exp(-k (|x - c| - R)) (x - c)/|x - c| at the four-point Gauss rule (the kernel's
// coordinates 0.58541020 / 0.13819669), distributed with the linear shape functions and weighted
// by |det[p1-p4, p2-p4, p3-p4]| / 4 (the current, deformed tetra). Corner positions relative to
// the centre and the edges are formed from the hi/lo parts of X and u, so large coordinates lose
// no precision. Adds the corner forces to the tetra's slots when s_cf is given; returns the sum
// of their y components (the readout's share).
template <int TILE>
__device__ __forceinline__ float sphere_integral(int j, uchar4 lc, const float4* s_uh, const float4* s_ul,
                                                 const float4* s_xh, const float4* s_xl, const SphereIntegralStep& sp,
                                                 float4* s_cf) {
    const int li[4] = {lc.x, lc.y, lc.z, lc.w};
    float4 xh[4], xl[4], uh[4], ul[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        xh[a] = s_xh[li[a]];
        xl[a] = s_xl[li[a]];
        uh[a] = s_uh[li[a]];
        ul[a] = s_ul[li[a]];
    }
    float d[4][3];  // corner minus sphere centre (0, cy, 0)
    float e[3][3];  // corners 1..3 minus corner 4
#pragma unroll
    for (int a = 0; a < 4; a++) {
        d[a][0] = (xh[a].x + uh[a].x) + (xl[a].x + ul[a].x);
        d[a][1] = ((xh[a].y - sp.cy_hi) + uh[a].y) + ((xl[a].y - sp.cy_lo) + ul[a].y);
        d[a][2] = (xh[a].z + uh[a].z) + (xl[a].z + ul[a].z);
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        e[a][0] = ((xh[a].x - xh[3].x) + (uh[a].x - uh[3].x)) + ((xl[a].x - xl[3].x) + (ul[a].x - ul[3].x));
        e[a][1] = ((xh[a].y - xh[3].y) + (uh[a].y - uh[3].y)) + ((xl[a].y - xl[3].y) + (ul[a].y - ul[3].y));
        e[a][2] = ((xh[a].z - xh[3].z) + (uh[a].z - uh[3].z)) + ((xl[a].z - xl[3].z) + (ul[a].z - ul[3].z));
    }
    const float cx = e[1][1] * e[2][2] - e[1][2] * e[2][1];
    const float cyv = e[1][2] * e[2][0] - e[1][0] * e[2][2];
    const float cz = e[1][0] * e[2][1] - e[1][1] * e[2][0];
    const float w = 0.25f * fabsf(e[0][0] * cx + e[0][1] * cyv + e[0][2] * cz);
    const float al = 0.58541020f, be = 0.13819669f;
    float F[4][3] = {};
#pragma unroll
    for (int g = 0; g < 4; g++) {
        float N[4];
        N[0] = g == 0 ? al : be;
        N[1] = g == 1 ? al : be;
        N[2] = g == 2 ? al : be;
        N[3] = 1.0f - N[0] - N[1] - N[2];
        float r[3];
#pragma unroll
        for (int q = 0; q < 3; q++) r[q] = N[0] * d[0][q] + N[1] * d[1][q] + N[2] * d[2][q] + N[3] * d[3][q];
        const float len = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const float mag = expf(-sp.k * (len - sp.radius)) / len;
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int q = 0; q < 3; q++) F[a][q] += (mag * N[a]) * r[q];
    }
    float fy = 0.f;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const float3 Fa = make_float3(w * F[a][0], w * F[a][1], w * F[a][2]);
        fy += Fa.y;
        if (s_cf) {
            float4 c = s_cf[a * TILE + j];
            c.x += Fa.x;
            c.y += Fa.y;
            c.z += Fa.z;
            s_cf[a * TILE + j] = c;
        }
    }
    return fy;
}

// Fixed-order sum of one float per thread of a CTA of TILE threads (shuffle tree, then the warps
// in order by thread 0), in double; every thread must call it. Returns the total on thread 0.
template <int TILE>
__device__ __forceinline__ double tile_sum(float v, double* s_scratch) {
    double x = (double)v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) s_scratch[threadIdx.x >> 5] = x;
    __syncthreads();
    double tot = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < TILE / 32; w++) tot += s_scratch[w];
    return tot;
}

// ------------------------------------------------------------------------------------------
// Element pass, one CTA per tile (plain loads)
// ------------------------------------------------------------------------------------------
// The tile's material comes from its cell's entry in the cell table (cell 0 when the table has
// no tile map), so a single simulation and a batch run this same code.
#ifndef NFX_TET_REGS
#define NFX_TET_REGS 56  // registers per thread of the element pass: 9 CTAs of 128 per SM (64: 8)
#endif
#ifndef NFX_DMI_FROM_X
#define NFX_DMI_FROM_X 0  // 1: Dm^-1 and V0 from the staged reference positions instead of the stored arrays
#endif

// Dm^-1 (row-major, in the stored arrays' layout) and V0 = det(Dm)/6 of one tetra from its
// corners' reference positions X = Xh + Xl staged in shared memory: Dm's columns are the edges
// X_k - X_0 (hi and lo parts differenced separately), the inverse is adj(Dm)/det(Dm) with a
// correctly rounded reciprocal — the host's construction in float.
__device__ __forceinline__ void ref_shape_inverse(uchar4 lc, const float4* s_xh, const float4* s_xl, float4& da,
                                                  float4& db, float2& dc) {
    const float4 h0 = s_xh[lc.x], l0 = s_xl[lc.x];
    const int lk[3] = {lc.y, lc.z, lc.w};
    float M[9];  // M[3 d + k] = X_(k+1),d - X_0,d
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float4 h = s_xh[lk[k]], l = s_xl[lk[k]];
        M[k] = (h.x - h0.x) + (l.x - l0.x);
        M[3 + k] = (h.y - h0.y) + (l.y - l0.y);
        M[6 + k] = (h.z - h0.z) + (l.z - l0.z);
    }
    const float A0 = M[4] * M[8] - M[5] * M[7], A1 = M[2] * M[7] - M[1] * M[8], A2 = M[1] * M[5] - M[2] * M[4];
    const float A3 = M[5] * M[6] - M[3] * M[8], A4 = M[0] * M[8] - M[2] * M[6], A5 = M[2] * M[3] - M[0] * M[5];
    const float A6 = M[3] * M[7] - M[4] * M[6], A7 = M[1] * M[6] - M[0] * M[7], A8 = M[0] * M[4] - M[1] * M[3];
    const float det = M[0] * A0 + M[1] * A3 + M[2] * A6;
    const float r = __frcp_rn(det);
    da = make_float4(A0 * r, A1 * r, A2 * r, A3 * r);
    db = make_float4(A4 * r, A5 * r, A6 * r, A7 * r);
    dc = make_float2(A8 * r, det * (1.0f / 6.0f));
}
// Tile-relative displacements: the element pass stages, per tile node, the displacement minus
// that of the tile's first node, (h - h_ref) + (l - l_ref) per component with u = h + l (hi/lo),
// in one float4 — a quantity of the size of the tile's deformation, which FP32 holds to the
// accuracy the hi/lo pair gives the differences — and a tetrahedron's edge differences are
// v_k - v_0. Against staging hi and lo (two float4 per node, and per corner two shared loads and
// nine additions), this halves the shared-memory traffic of the gather, the pass's busiest unit.
#ifndef NFX_TILE_REL
#define NFX_TILE_REL 1
#endif
template <int MODEL, int TILE>
__device__ __forceinline__ bool element_eval_rel(int j, long long t, uchar4 lc, float4 da, float4 db, float2 dc,
                                                 float4 pa, float4 pb, float2 pc, const float4* s_v, float4* s_cf,
                                                 const StateDev& s, const MaterialDev& mat, bool write_fields) {
    const int li[4] = {lc.x, lc.y, lc.z, lc.w};
    const float4 v0 = s_v[li[0]];
    float d[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float4 v = s_v[li[k + 1]];
        d[k][0] = v.x - v0.x;
        d[k][1] = v.y - v0.y;
        d[k][2] = v.z - v0.z;
    }
    return element_law<MODEL, TILE>(j, t, d, da, db, dc, pa, pb, pc, s_cf, s, mat, write_fields);
}

template <int MODEL, int TILE>
__global__ void __launch_bounds__(TILE, 65536 / (TILE * NFX_TET_REGS))
    k_tet_pass(MeshDev m, StateDev s, BatchDev bd, int t_offset) {
    constexpr int NMAX = TILE < TILE_NODES_MAX ? TILE : TILE_NODES_MAX;
#if NFX_TILE_REL
    __shared__ float4 s_v[NMAX];  // tile-relative displacement of each tile node (x, y, z)
#else
    __shared__ float4 s_uh[NMAX];
    __shared__ float4 s_ul[NMAX];
#endif
    __shared__ float4 s_cf[4 * TILE];  // corner forces, slot corner*TILE + local tet
    __shared__ ushort4 s_inc[TILE];    // the tile's incidence list
#if NFX_DMI_FROM_X
    __shared__ float4 s_xh[NMAX];
    __shared__ float4 s_xl[NMAX];
#endif

    // Serpentine order across the kernel boundaries: the node pass runs its blocks in ascending
    // node order, the element pass its tiles in descending order, so each pass starts on the nodes
    // (accumulator words, displacements) the previous pass touched last and that are still in L2.
    // The order changes no result: tile sums enter the accumulator as integers.
#ifndef NFX_TILE_REVERSE
#define NFX_TILE_REVERSE 1
#endif
#if NFX_PDL_TET
    grid_dep_wait();  // the node pass (or whatever preceded) has completed
#endif
    const int b = NFX_TILE_REVERSE ? (int)(gridDim.x - 1 - blockIdx.x) : (int)blockIdx.x;
    const int j = threadIdx.x;
#if NFX_TET_TRIGGER
    if (j == 0) grid_dep_trigger();
#endif
    // fixed-stride tiles: the tile's slots and node entries are addressed without a load; the
    // real counts come from the tile's meta word (loaded alongside the data)
    const int t = b * TILE + j;
    const int nb = b * NMAX;
    const unsigned meta = __ldg(m.tile_meta + b);
    const int ntt = (int)(meta & 0xffffu);
    const int nn = (int)(meta >> 16);
    const bool act = j < ntt;
    const bool wf = clock_bit(s.clock->fields_due, t_offset);

    // Streaming per-tetra data (read once per step: evict-first) and the node list, issued for
    // every slot and entry without waiting for the meta word: padding is valid zeroed memory.
    const uchar4 lc = __ldcs(m.lconn + t);
#if !NFX_DMI_FROM_X
    const float4 da = __ldcs(m.dmi_a + t);
    const float4 db = __ldcs(m.dmi_b + t);
    const float2 dc = __ldcs(m.dmi_c + t);
#endif
    float4 pa = make_float4(0.f, 0.f, 0.f, 0.f), pb = pa;
    float2 pc = make_float2(0.f, 0.f);
    if (MODEL == MODEL_VP) {
        pa = __ldcs(s.vp_a + t);
        pb = __ldcs(s.vp_b + t);
        pc = __ldcs(s.vp_c + t);
    }
    s_inc[j] = __ldcs(m.tile_inc + t);
    uint2 node = make_uint2(0u, 0u);
#if NFX_TILE_REL
    // the tile's first node (every thread loads the same words: one broadcast transaction)
    const unsigned ref = __ldg(&m.tile_nodes[nb].x);
    const float4 ar = s.ua[ref];
    const float2 lr = s.ub[ref];
#endif
    if (j < NMAX) {
        node = __ldcs(m.tile_nodes + nb + j);
        const float4 a = s.ua[node.x];
        const float2 lo = s.ub[node.x];
#if NFX_TILE_REL
        s_v[j] = make_float4((a.x - ar.x) + (a.w - ar.w), (a.y - ar.y) + (lo.x - lr.x), (a.z - ar.z) + (lo.y - lr.y),
                             0.f);
#else
        s_uh[j] = a;  // the law reads x, y, z only
        s_ul[j] = make_float4(a.w, lo.x, lo.y, 0.f);
#endif
#if NFX_DMI_FROM_X
        s_xh[j] = m.Xh[node.x];
        s_xl[j] = m.Xl[node.x];
#endif
    }
    const MaterialDev mat = bd.cells[bd.tile_cell ? __ldg(bd.tile_cell + b) : 0].mat;
    __syncthreads();
#if NFX_DMI_FROM_X
    float4 da = make_float4(0.f, 0.f, 0.f, 0.f), db = da;
    float2 dc = make_float2(0.f, 0.f);
    if (act) ref_shape_inverse(lc, s_xh, s_xl, da, db, dc);
#endif
#if NFX_TILE_REL
    if (act && element_eval_rel<MODEL, TILE>(j, t, lc, da, db, dc, pa, pb, pc, s_v, s_cf, s, mat, wf))
        raise_status(s, tile_cell_status(bd, b), STATUS_INVERTED);
#else
    if (act && element_eval<MODEL, TILE>(j, t, lc, da, db, dc, pa, pb, pc, s_uh, s_ul, s_cf, s, mat, wf))
        raise_status(s, tile_cell_status(bd, b), STATUS_INVERTED);
#endif
    __syncthreads();
    if (j < nn && !node_flush<TILE>(node, reinterpret_cast<const unsigned short*>(s_inc), s_cf, s, m.np, m.fix_max))
        raise_status(s, tile_cell_status(bd, b), STATUS_NONFINITE);
}

// Integrated sphere contact (InteractionSphereIntegral.cl), one CTA per tile of a cell that has
// one; tiles of other cells return at once. SI_STEP: inside a step (time offset t_offset) — the
// sphere's corner forces are summed per tile node in the tile's fixed incidence order and added
// to the force accumulator like the element pass's, and on record steps of that contact the
// tile's share of the readout (sum of the y forces) goes to tile_partials. SI_READOUT: only the
// readout shares of contact index `contact` at the current positions (readouts between steps).
enum SiMode : int { SI_STEP = 0, SI_READOUT = 1 };
template <int TILE>
__global__ void __launch_bounds__(TILE) k_si_pass(MeshDev m, StateDev s, BatchDev bd, int t_offset, int mode,
                                                  int contact) {
    constexpr int NMAX = TILE < TILE_NODES_MAX ? TILE : TILE_NODES_MAX;
    __shared__ float4 s_uh[NMAX], s_ul[NMAX], s_xh[NMAX], s_xl[NMAX];
    __shared__ float4 s_cf[4 * TILE];
    __shared__ ushort4 s_inc[TILE];
    __shared__ SphereIntegralStep s_sp;
    __shared__ double s_red[TILE / 32];
    const int b = blockIdx.x, j = threadIdx.x;
    const int cell = bd.tile_cell ? __ldg(bd.tile_cell + b) : 0;
    const CellDev& C = bd.cells[cell];
    const int si = C.si_contact;
    if (si < 0 || (mode == SI_READOUT && si != contact)) return;  // uniform over the CTA
    const int t = b * TILE + j;
    const unsigned meta = __ldg(m.tile_meta + b);
    const int ntt = (int)(meta & 0xffffu), nn = (int)(meta >> 16);
    uint2 node = make_uint2(0u, 0u);
    if (j < NMAX) {
        node = m.tile_nodes[b * NMAX + j];
        const float4 a = s.ua[node.x];
        const float2 lo = s.ub[node.x];
        s_uh[j] = a;
        s_ul[j] = make_float4(a.w, lo.x, lo.y, 0.f);
        s_xh[j] = m.Xh[node.x];
        s_xl[j] = m.Xl[node.x];
    }
    const uchar4 lc = m.lconn[t];
    if (mode == SI_STEP) s_inc[j] = m.tile_inc[t];
    const long long time = s.clock->time + (mode == SI_STEP ? t_offset : 0);
    if (j == 0) {
        const double cy = contact_pos(C.c[si], time);
        const float hi = (float)cy;
        s_sp = SphereIntegralStep{hi, (float)(cy - (double)hi), (float)C.c[si].radius, (float)C.c[si].k};
    }
#pragma unroll
    for (int a = 0; a < 4; a++) s_cf[a * TILE + j] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const float fy = j < ntt ? sphere_integral<TILE>(j, lc, s_uh, s_ul, s_xh, s_xl, s_sp, s_cf) : 0.f;
    const bool want_partial =
        mode == SI_READOUT || (si == C.record_contact && clock_bit(s.clock->record_due, t_offset));
    if (want_partial) {  // uniform over the CTA
        const double tot = tile_sum<TILE>(fy, s_red);
        if (j == 0) s.tile_partials[m.tile_base + b] = tot;
    }
    if (mode != SI_STEP) return;
    __syncthreads();
    if (j < nn && !node_flush<TILE>(node, reinterpret_cast<const unsigned short*>(s_inc), s_cf, s, m.np, m.fix_max))
        raise_status(s, bd.cell_status ? bd.cell_status + cell : nullptr, STATUS_NONFINITE);
}

// ------------------------------------------------------------------------------------------
// Node pass
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// A contact's values for one step, shared by a node block: the position in double for the
// exact formulas, and in float (with the sphere radius) for the coarse test every node runs, so
// that no node converts a double (conversions run on the FP64 pipe).
struct WallStep {
    double w;
    float wf, rf;
};

// Whether a contact can reach a node, from its node block's reference box (lo, hi: the bounding
// box of the block's reference positions, rounded outwards) shifted by the node's own
// displacement hi part: the coarse test of contact_force (substrate: y < w + 1e-3, plane:
// y > w - 1e-3, sphere: within radius + 1e-3 of (0, w, 0)) applied to that box, widened by a
// further margin that covers the float rounding of the node's coarse position x_hi + u_hi (a few
// ulps of the coordinates) many times over. A node it rejects would fail the coarse test too, so
// the node's reference position (16 bytes) is read only where a contact may act on the node.
#ifndef NFX_NODE_CULL
#define NFX_NODE_CULL 1  // 0: every node reads its reference position
#endif
// Whether a node block lies within EAGER_REACH lattice units of a contact, judged on its reference
// box alone (a heuristic for when to read reference positions early; the per-node test above
// decides what is evaluated, so the answer never changes a result).
constexpr float EAGER_REACH = 4.0f;
__device__ __forceinline__ bool block_near(const ContactDev* cs, int nc, const WallStep* wall, float4 lo, float4 hi) {
    bool near = false;
    for (int c = 0; c < nc; c++) {
        const ContactDev& k = cs[c];
        const float wf = wall[c].wf;
        if (k.kind == CONTACT_SUBSTRATE) {
            near |= lo.y - EAGER_REACH < wf;
        } else if (k.kind == CONTACT_PLANE) {
            near |= hi.y + EAGER_REACH > wf;
        } else if (k.kind == CONTACT_SPHERE) {
            const float dx = fmaxf(fmaxf(lo.x, -hi.x), 0.f), dy = fmaxf(fmaxf(lo.y - wf, wf - hi.y), 0.f),
                        dz = fmaxf(fmaxf(lo.z, -hi.z), 0.f);
            const float r = wall[c].rf + EAGER_REACH;
            near |= dx * dx + dy * dy + dz * dz < r * r;
        }
    }
    return near;
}

__device__ __forceinline__ bool contact_reaches(const ContactDev& c, const WallStep& ws, float4 lo, float4 hi,
                                                const float4& uh) {
    if (c.kind == CONTACT_SPHERE_INTEGRAL) return false;  // a per-tetra force (element pass)
    if (!NFX_NODE_CULL) return true;
    const float M = 2e-3f;
    if (c.kind == CONTACT_SUBSTRATE) return !((lo.y + uh.y) - M > ws.wf);
    if (c.kind == CONTACT_PLANE) return !((hi.y + uh.y) + M < ws.wf);
    const float dx = fmaxf(fmaxf(lo.x + uh.x, -(hi.x + uh.x)), 0.f);
    const float dy = fmaxf(fmaxf((lo.y + uh.y) - ws.wf, ws.wf - (hi.y + uh.y)), 0.f);
    const float dz = fmaxf(fmaxf(lo.z + uh.z, -(hi.z + uh.z)), 0.f);
    const float r = ws.rf + M;
    return !(dx * dx + dy * dy + dz * dz > r * r);
}

// The exact contact force (the reference's FP64 formulas) on one node that passed the coarse
// float test. Every double term is formed after the low-part load, so none of the double
// arithmetic can be hoisted above the coarse test: with the terms of (x_hi + x_lo) + (u_hi + u_lo)
// independent of that load, the compiler ran the displacement sums for every node (about three
// DADDs per node on the narrow FP64 pipe). hit = false: the node does not touch (sphere only).
struct ContactForce {
    double fx, fy, fz;
    bool hit;
};
__device__ __forceinline__ ContactForce contact_exact(const ContactDev& c, double w, float4 xh, float4 xl, float4 uh,
                                                      float4 ul) {
    ContactForce r{0.0, 0.0, 0.0, true};
    const double y = (((double)xh.y + (double)xl.y) + (double)uh.y) + (double)ul.y;
    if (c.kind == CONTACT_SUBSTRATE || c.kind == CONTACT_PLANE) {
        r.fy = c.kind == CONTACT_SUBSTRATE ? c.k * fmax(w - y, 0.0) : -c.k * fmax(y - w, 0.0);
        return r;
    }
    // sphere centred at (0, w, 0)
    const double rx = (((double)xh.x + (double)xl.x) + (double)uh.x) + (double)ul.x;
    const double ry = y - w;
    const double rz = (((double)xh.z + (double)xl.z) + (double)uh.z) + (double)ul.z;
    const double len = sqrt(rx * rx + ry * ry + rz * rz);
    const double dis = fmax(c.radius - len, 0.0);
    if (dis == 0.0) {
        r.hit = false;
        return r;
    }
    const double kd = c.k * dis;
    r.fx = kd * (rx / len);
    r.fy = kd * (ry / len);
    r.fz = kd * (rz / len);
    return r;
}

// Contact force on one node: the coarse test in float (nodes farther than 1e-3 from contact
// cannot touch), then the exact force. Returns false for a node out of contact; otherwise adds
// the force to f and returns its y component in fy for the readout.
__device__ __forceinline__ bool contact_force(const ContactDev& c, const WallStep& ws, const float4& xh,
                                              const float4* xlp, const float4& uh, const float4& ul, float4& f,
                                              double& fy) {
    if (c.kind == CONTACT_SPHERE_INTEGRAL) return false;  // a per-tetra force (element pass)
    const float yf = xh.y + uh.y;
    if (c.kind == CONTACT_SUBSTRATE) {
        if (ws.wf - yf < -1e-3f) return false;
    } else if (c.kind == CONTACT_PLANE) {
        if (yf - ws.wf < -1e-3f) return false;
    } else {
        const float rxf = xh.x + uh.x, ryf = yf - ws.wf, rzf = xh.z + uh.z;
        const float rr = ws.rf + 1e-3f;
        if (rxf * rxf + ryf * ryf + rzf * rzf > rr * rr) return false;
    }
    const ContactForce r = contact_exact(c, ws.w, xh, *xlp, uh, ul);
    if (!r.hit) return false;
    if (c.kind == CONTACT_SPHERE) {
        f.x += (float)r.fx;
        f.z += (float)r.fz;
    }
    f.y += (float)r.fy;
    fy = r.fy;
    return true;
}

// One node, in two halves. node_load reads the displacement hi/lo and, in a block near a
// contact, the reference position. node_finish adds the element force from the fixed-point
// accumulator and the contacts in order (returning the y force of contact rc on the node; the
// readout is minus its sum, negated once per cell so that no node runs a double negation), and in
// update mode runs the cell's integrator with the displacement carried as hi + lo — damped
// velocity Verlet with unit mass and the FIXED_TOP_BOTTOM pin (VelocityVerlet.cl), or the
// lumped-mass form (velocityVerlet2.cl) — and resets the accumulator.
struct NodeLoad {
    float4 xh, a;  // reference position (when loaded), displacement hi + u_lo.x
    float2 lo;     // u_lo.yz
    bool xh_loaded;
};
__device__ __forceinline__ NodeLoad node_load(const MeshDev& m, const StateDev& s, int i, bool near,
                                              const CellDev& C) {
    NodeLoad r;
    // In a block near a contact (or under the lumped-mass integrator, which needs Xh.w) the
    // reference position is read with the node's first loads; elsewhere only after the per-node
    // test in node_finish says a contact can reach the node.
    r.xh_loaded = near || C.integrator == INTEGRATOR_VV2;
    r.xh = make_float4(0.f, 0.f, 0.f, 0.f);
    if (r.xh_loaded) r.xh = m.Xh[i];
    r.a = s.ua[i];
    r.lo = s.ub[i];
    return r;
}

__device__ __forceinline__ double node_finish(const MeshDev& m, const StateDev& s, int i, const WallStep* wall,
                                              const float4* box, const NodeLoad& L, const CellDev& C, int rc,
                                              bool update, unsigned* cstat) {
    const ContactDev* cs = C.c;
    const int nc = C.n_contacts;
    const long long np = m.np;
    float4 f = make_float4(fix_to_float(s.facc[i]), fix_to_float(s.facc[np + i]), fix_to_float(s.facc[2 * np + i]), 0.f);
    float4 uh = make_float4(L.a.x, L.a.y, L.a.z, 0.f), ul = make_float4(L.a.w, L.lo.x, L.lo.y, 0.f);
    float4 xh = L.xh;
    // the contacts that may act on this node; the reference position only where one may, or where
    // the lumped-mass integrator needs the inverse mass (Xh.w)
    unsigned reach = 0u;
    const float4 blo = box[0], bhi = box[1];
    for (int c = 0; c < nc; c++)
        if (contact_reaches(cs[c], wall[c], blo, bhi, uh)) reach |= 1u << c;
    if (!L.xh_loaded && reach) xh = m.Xh[i];
    double fy_rc = 0.0;
    for (int c = 0; c < nc; c++) {
        double fy;
        if (((reach >> c) & 1u) && contact_force(cs[c], wall[c], xh, m.Xl + i, uh, ul, f, fy) && c == rc) fy_rc = fy;
    }
    if (!update) return fy_rc;
    // velocity and previous force: streamed once per step (evict-first)
    const float4 va = __ldcs(s.va + i);
    const float2 vb = __ldcs(s.vb + i);
    float3 v = make_float3(va.x, va.y, va.z);
    float3 nf;  // the new previous-force slot
    if (C.integrator == INTEGRATOR_VV2) {
        // velocityVerlet2.cl:9-13: v = (v + (a_old + f/m)/2) / (1 + xi/2); a = f/m - xi v;
        // x += v + a/2; the old-force slot keeps a
        const float minv = xh.w * C.inv_density;
        const float c = C.vv2_c, xi = C.vv2_xi;
        const float fx = f.x * minv, fy = f.y * minv, fz = f.z * minv;
        v.x = c * (v.x + 0.5f * (va.w + fx));
        v.y = c * (v.y + 0.5f * (vb.x + fy));
        v.z = c * (v.z + 0.5f * (vb.y + fz));
        const float ax = fx - xi * v.x, ay = fy - xi * v.y, az = fz - xi * v.z;
        df_add(uh.x, ul.x, v.x + 0.5f * ax);
        df_add(uh.y, ul.y, v.y + 0.5f * ay);
        df_add(uh.z, ul.z, v.z + 0.5f * az);
        nf = make_float3(ax, ay, az);
    } else {
        const float vv_a = C.vv_a, vv_hb = C.vv_hb, vv_dm = C.vv_dm;
        v.x = vv_a * v.x + vv_hb * (f.x + va.w);
        v.y = vv_a * v.y + vv_hb * (f.y + vb.x);
        v.z = vv_a * v.z + vv_hb * (f.z + vb.y);
        df_add(uh.x, ul.x, vv_dm * v.x + 0.5f * f.x);
        df_add(uh.y, ul.y, vv_dm * v.y + 0.5f * f.y);
        df_add(uh.z, ul.z, vv_dm * v.z + 0.5f * f.z);
        if (i == C.fix_a || i == C.fix_b) {  // VelocityVerlet.cl:17-22: x = z = 0
            const float4 xp = m.Xh[i], xl = m.Xl[i];
            uh.x = -xp.x;
            ul.x = -xl.x;
            uh.z = -xp.z;
            ul.z = -xl.z;
        }
        nf = make_float3(f.x, f.y, f.z);
    }
    if (!isfinite(uh.x + uh.y + uh.z + v.x + v.y + v.z)) raise_status(s, cstat, STATUS_NONFINITE);
    s.ua[i] = make_float4(uh.x, uh.y, uh.z, ul.x);
    s.ub[i] = make_float2(ul.y, ul.z);
    __stcs(s.va + i, make_float4(v.x, v.y, v.z, nf.x));
    __stcs(s.vb + i, make_float2(nf.y, nf.z));
    s.facc[i] = 0ull;
    s.facc[np + i] = 0ull;
    s.facc[2 * np + i] = 0ull;
    return fy_rc;
}

// One thread per node. The block's cell (cell 0 without a block map) supplies the contacts and
// the integrator. On record steps (and for on-demand readouts) the readout values are summed per
// cell in a fixed order: warp shuffles, then the block's warps in order, then — by the cell's
// last block to finish — the cell's block partials in index order, so the result is the same on
// every run and does not depend on which other cells share the launch.
#ifndef NFX_NODE_MIN_BLOCKS
#define NFX_NODE_MIN_BLOCKS 4  // resident node-pass blocks per SM (64 registers; 4 cost 30 us less than 1 at R=64)
#endif
__global__ void __launch_bounds__(NODE_BLOCK, NFX_NODE_MIN_BLOCKS) k_node_pass(MeshDev m, StateDev s, BatchDev bd, int t_offset, int mode,
                                                          int readout_contact) {
    __shared__ double s_w[NODE_BLOCK / 32];
    __shared__ WallStep s_wall[MAX_CONTACTS];
    __shared__ float4 s_box[2];
    __shared__ int s_last;
#if NFX_PDL_TET
    if (threadIdx.x == 0) grid_dep_trigger();  // the next element pass may take freed SMs
#endif
    const int cell = bd.block_cell ? __ldg(bd.block_cell + blockIdx.x) : 0;
    const CellDev& C = bd.cells[cell];
    const int i = blockIdx.x * NODE_BLOCK + threadIdx.x;
    const long long t = s.clock->time + t_offset;
    // the cell's contact positions at time t, once per block (FP64 and table lookups stay off the
    // per-node path)
    if (threadIdx.x < C.n_contacts) {
        const double w = contact_pos(C.c[threadIdx.x], t);
        s_wall[threadIdx.x] = WallStep{w, (float)w, (float)C.c[threadIdx.x].radius};
    }
    if (threadIdx.x >= 32 && threadIdx.x < 34) s_box[threadIdx.x - 32] = m.block_box[2 * blockIdx.x + (threadIdx.x - 32)];
    __syncthreads();
#if NFX_PDL_NODE
    grid_dep_wait();  // the element pass's forces in the accumulator
#endif
    int rc;
    bool rec;
    long long row = 0;
    if (mode == NODE_READOUT_VALUE) {
        rc = readout_contact;
        rec = true;
    } else {
        rc = C.record_contact;
        rec = rc >= 0 && clock_bit(s.clock->record_due, t_offset);
        if (rec) {
            row = t / bd.record_every;
            if (row >= bd.max_rows) {
                if (threadIdx.x == 0) atomicOr(s.status, STATUS_CURVE_FULL);
                rec = false;
            }
        }
    }
    double fy = 0.0;  // y force of the readout contact on this node
    const bool update = mode == NODE_UPDATE;
    unsigned* cstat = bd.cell_status ? bd.cell_status + cell : nullptr;
    const bool near = !NFX_NODE_CULL || block_near(C.c, C.n_contacts, s_wall, s_box[0], s_box[1]);
    if (i < C.node_end) fy = node_finish(m, s, i, s_wall, s_box, node_load(m, s, i, near, C), C, rc, update, cstat);
    if (!rec) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    fy = warp_sum_d(fy);
    if (lane == 0) s_w[warp] = fy;
    __syncthreads();
    if (warp == 0) {
        double x = lane < NODE_BLOCK / 32 ? s_w[lane] : 0.0;
        x = warp_sum_d(x);
        if (lane == 0) {
            s.partials[blockIdx.x] = x;
            __threadfence();
            const unsigned prev = atomicAdd(bd.cell_counter + cell, 1u);
            s_last = prev == (unsigned)(C.block_end - C.block_begin - 1);
        }
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const volatile double* part = s.partials;
    double acc = 0.0;
    for (int k = C.block_begin + threadIdx.x; k < C.block_end; k += NODE_BLOCK) acc += part[k];
    if (rc >= 0 && rc == C.si_contact) {
        // integrated sphere: the y forces summed per tile by the element pass (or by the sphere
        // pass for an on-demand readout)
        const volatile double* tp = s.tile_partials;
        for (int k = C.tile_begin + threadIdx.x; k < C.tile_end; k += NODE_BLOCK) acc += tp[k];
    }
    acc = warp_sum_d(acc);
    if (lane == 0) s_w[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < NODE_BLOCK / 32; w++) sum += s_w[w];
        // the readout is minus the summed y force (negation is exact and rounding is symmetric,
        // so this equals summing the negated forces)
        const double tot = 0.0 - sum;
        if (mode == NODE_READOUT_VALUE) {
            s.force_out[cell] = tot;
        } else {
            double* r = bd.curves + 3 * ((long long)cell * bd.max_rows + row);
            r[0] = (double)t;
            r[1] = contact_pos(C.c[rc], 0) - s_wall[rc].w;
            r[2] = tot;
        }
        bd.cell_counter[cell] = 0u;
    }
}

// One block of CLOCK_WINDOW threads: thread k evaluates step time + k of the next window.
__global__ void __launch_bounds__(CLOCK_WINDOW) k_advance_time(StepClock* c, long long n, long long fields_every,
                                                               long long record_every) {
    const int k = threadIdx.x;
    const long long t0 = c->time + n;
    const long long t = t0 + k;
    const bool f = fields_every > 0 && (t + 1) % fields_every == 0;
    const bool r = record_every > 0 && t % record_every == 0;
    const unsigned fm = __ballot_sync(0xffffffffu, f), rm = __ballot_sync(0xffffffffu, r);
    __syncthreads();  // every thread has read the old time
    if ((k & 31) == 0) {
        c->fields_due[k >> 5] = fm;
        c->record_due[k >> 5] = rm;
    }
    if (k == 0) c->time = t0;
}

// ------------------------------------------------------------------------------------------
// Layout conversions (user order, SoA doubles) <-> device state
// ------------------------------------------------------------------------------------------
__global__ void k_points_to_user(MeshDev m, StateDev s, const long long* node_user, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.np) return;
    const long long u = node_user[i];
    const float4 xh = m.Xh[i], xl = m.Xl[i], uh = s.ua[i];
    const float2 lo = s.ub[i];
    const float4 ul = make_float4(uh.w, lo.x, lo.y, 0.f);
    out[u] = ((double)xh.x + (double)xl.x) + ((double)uh.x + (double)ul.x);
    out[m.np + u] = ((double)xh.y + (double)xl.y) + ((double)uh.y + (double)ul.y);
    out[2 * (long long)m.np + u] = ((double)xh.z + (double)xl.z) + ((double)uh.z + (double)ul.z);
}

__global__ void k_points_from_user(MeshDev m, StateDev s, const long long* node_user, const double* in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.np) return;
    const long long u = node_user[i];
    const float4 xh = m.Xh[i], xl = m.Xl[i];
    const double dx = (in[u] - (double)xh.x) - (double)xl.x;
    const double dy = (in[m.np + u] - (double)xh.y) - (double)xl.y;
    const double dz = (in[2 * (long long)m.np + u] - (double)xh.z) - (double)xl.z;
    const float hx = (float)dx, hy = (float)dy, hz = (float)dz;
    s.ua[i] = make_float4(hx, hy, hz, (float)(dx - hx));
    s.ub[i] = make_float2((float)(dy - hy), (float)(dz - hz));
}

// part 0: (a.x, a.y, a.z); part 1: (a.w, b.x, b.y)
__global__ void k_vec_to_user(int np, const float4* a, const float2* b, int part, const long long* node_user,
                              double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const long long u = node_user[i];
    const float4 q = a[i];
    float x = q.x, y = q.y, z = q.z;
    if (part == 1) {
        const float2 r = b[i];
        x = q.w;
        y = r.x;
        z = r.y;
    }
    out[u] = x;
    out[np + u] = y;
    out[2 * (long long)np + u] = z;
}

__global__ void k_vec_from_user(int np, float4* a, float2* b, int part, const long long* node_user,
                                const double* in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const long long u = node_user[i];
    const float x = (float)in[u], y = (float)in[np + u], z = (float)in[2 * (long long)np + u];
    float4 q = a[i];
    if (part == 0) {
        q.x = x;
        q.y = y;
        q.z = z;
    } else {
        q.w = x;
        b[i] = make_float2(y, z);
    }
    a[i] = q;
}

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------
template <int MODEL, int TILE>
static cudaError_t launch_tet(const MeshDev& m, const StateDev& s, const BatchDev& b, int t_offset, cudaStream_t st,
                              bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)m.ntiles);
    cfg.blockDim = dim3(TILE);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (NFX_PDL_TET && pdl) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_tet_pass<MODEL, TILE>, m, s, b, t_offset);
}

template <int TILE>
static cudaError_t launch_tile(const MeshDev& m, const StateDev& s, const BatchDev& b, int model, int t_offset,
                               cudaStream_t st, bool pdl) {
    switch (model) {
        case MODEL_MR: return launch_tet<MODEL_MR, TILE>(m, s, b, t_offset, st, pdl);
        case MODEL_SVK: return launch_tet<MODEL_SVK, TILE>(m, s, b, t_offset, st, pdl);
        case MODEL_SVKK: return launch_tet<MODEL_SVKK, TILE>(m, s, b, t_offset, st, pdl);
        case MODEL_VP: return launch_tet<MODEL_VP, TILE>(m, s, b, t_offset, st, pdl);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_tet_pass(const MeshDev& m, const StateDev& s, const BatchDev& b, int model, int t_offset,
                            cudaStream_t st, bool pdl) {
    if (m.ntiles <= 0) return cudaSuccess;
    switch (m.tile_tets) {
        case 64: return launch_tile<64>(m, s, b, model, t_offset, st, pdl);
        case 128: return launch_tile<128>(m, s, b, model, t_offset, st, pdl);
        case 256: return launch_tile<256>(m, s, b, model, t_offset, st, pdl);
        case 512: return launch_tile<512>(m, s, b, model, t_offset, st, pdl);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_si_pass(const MeshDev& m, const StateDev& s, const BatchDev& b, int t_offset, bool readout,
                          int contact, cudaStream_t st) {
    if (m.ntiles <= 0) return cudaSuccess;
    const int mode = readout ? SI_READOUT : SI_STEP;
    switch (m.tile_tets) {
        case 64: k_si_pass<64><<<m.ntiles, 64, 0, st>>>(m, s, b, t_offset, mode, contact); break;
        case 128: k_si_pass<128><<<m.ntiles, 128, 0, st>>>(m, s, b, t_offset, mode, contact); break;
        case 256: k_si_pass<256><<<m.ntiles, 256, 0, st>>>(m, s, b, t_offset, mode, contact); break;
        case 512: k_si_pass<512><<<m.ntiles, 512, 0, st>>>(m, s, b, t_offset, mode, contact); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_node_pass(const MeshDev& m, const StateDev& s, const BatchDev& b, int nblocks, int t_offset,
                             int mode, int readout_contact, cudaStream_t st, bool pdl) {
    if (nblocks <= 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)nblocks);
    cfg.blockDim = dim3(NODE_BLOCK);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (NFX_PDL_NODE && pdl) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_node_pass, m, s, b, t_offset, mode, readout_contact);
}

cudaError_t launch_advance_time(const StateDev& s, long long n, long long fields_every, long long record_every,
                                cudaStream_t st) {
    k_advance_time<<<1, CLOCK_WINDOW, 0, st>>>(s.clock, n, fields_every, record_every);
    return cudaGetLastError();
}

cudaError_t launch_points_to_user(const MeshDev& m, const StateDev& s, const long long* node_user, double* out,
                                  cudaStream_t st) {
    k_points_to_user<<<(m.np + 255) / 256, 256, 0, st>>>(m, s, node_user, out);
    return cudaGetLastError();
}

__global__ void k_divide_check(const float* a, const float* b, float* q, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = fdiv_(a[i], b[i]);
}

cudaError_t launch_divide_check(const float* a, const float* b, float* q, long long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_divide_check<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, b, q, n);
    return cudaGetLastError();
}

cudaError_t launch_points_from_user(const MeshDev& m, const StateDev& s, const long long* node_user,
                                    const double* in, cudaStream_t st) {
    k_points_from_user<<<(m.np + 255) / 256, 256, 0, st>>>(m, s, node_user, in);
    return cudaGetLastError();
}

cudaError_t launch_vec_to_user(const MeshDev& m, const float4* a, const float2* b, int part, const long long* node_user,
                               double* out, cudaStream_t st) {
    k_vec_to_user<<<(m.np + 255) / 256, 256, 0, st>>>(m.np, a, b, part, node_user, out);
    return cudaGetLastError();
}

cudaError_t launch_vec_from_user(const MeshDev& m, float4* a, float2* b, int part, const long long* node_user,
                                 const double* in, cudaStream_t st) {
    k_vec_from_user<<<(m.np + 255) / 256, 256, 0, st>>>(m.np, a, b, part, node_user, in);
    return cudaGetLastError();
}

}  // namespace nfx
