// Per-element and per-node arithmetic of the noFluidX3D tetra step, in FP32.
//
// The formulas are the reference's (cited per function), rewritten so that FP32 keeps the
// accuracy the reference gets from FP64:
//  * strains come from displacement differences: with u = x - X the displacement gradient is
//    H = [u1-u0, u2-u0, u3-u0] * Dm^-1 and F = I + H; B - I = H + H^T + H H^T and
//    det F - 1 = tr H + i2(H) + det H are formed from small quantities only, so no
//    O(1) term is subtracted from another (the reference forms F = rT * J^-1 from absolute
//    positions, tetra.cl:37-63, which in FP32 leaves 6e-8 absolute noise in the strain);
//  * the Cauchy stress of the compressible Mooney-Rivlin law (tetra.cl:140-156) is expanded
//    in E = B - I;
//  * the nodal forces use inv(rT) = Dm^-1 F^-1 (tetra.cl:159-162): rows of
//    -V0 * Dm^-1 * adj(F) * sigma, with adj(F) = det(F) F^-1.
// All functions are __host__ __device__ so the arithmetic has one definition.
#pragma once

#if defined(__CUDACC__)
#define NFX_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define NFX_HD inline
#endif

namespace nfx {

#if defined(__CUDACC__)
NFX_HD float rcbrt_(float x) {
#if defined(__CUDA_ARCH__)
    return rcbrtf(x);
#else
    return 1.0f / cbrtf(x);
#endif
}
NFX_HD float pow_(float x, float y) { return powf(x, y); }
NFX_HD float sqrt_(float x) { return sqrtf(x); }
// a / b for the element laws. The fast reciprocal-based divide (__fdividef, up to 2 ulp) is
// refined by Markstein's method (P. Markstein, "IA-64 and Elementary Functions", 2000): one
// Newton-Raphson step on the reciprocal, r' = r + r (1 - b r), then the quotient corrected by its
// exact residual, q' = q + r' (a - b q), each residual a single fused multiply-add. Four FMAs and
// no branch; the result agrees with the correctly rounded quotient to within 1 ulp (checked
// against a / b on the GPU in the tests). The plastic state integrates quotients over every step,
// and the fast divide's bias alone moved the 10^4-step viscoplastic force curve by 1e-5.
// Valid for normal |b| below 2^126 (the element laws divide by determinants and stresses).
#ifndef NFX_DIV_REFINE
#define NFX_DIV_REFINE 1  // 0: the fast divide alone
#endif
NFX_HD float fdiv_(float a, float b) {
#if defined(__CUDA_ARCH__)
    float r = __fdividef(1.0f, b);
#if NFX_DIV_REFINE
    r = fmaf(r, fmaf(-b, r, 1.0f), r);
    const float q = a * r;
    return fmaf(r, fmaf(-b, q, a), q);
#else
    return a * r;
#endif
#else
    return a / b;
#endif
}
#else
NFX_HD float rcbrt_(float x) { return 1.0f / std::cbrt(x); }
NFX_HD float pow_(float x, float y) { return std::pow(x, y); }
NFX_HD float sqrt_(float x) { return std::sqrt(x); }
NFX_HD float fdiv_(float a, float b) { return a / b; }
#endif

// Symmetric 3x3 stored as (xx, yy, zz, xy, yz, xz).
struct Sym3 {
    float xx, yy, zz, xy, yz, xz;
};

// Row-major 3x3.
struct Mat3 {
    float m[9];
};

NFX_HD float tr(const Mat3& a) { return a.m[0] + a.m[4] + a.m[8]; }

// Displacement gradient H = Du * Dmi with Du's columns d1, d2, d3 (d_k = u_k - u_0) and Dmi
// the inverse reference edge matrix, row-major (Dmi[3k+j] = (Dm^-1)_kj).
NFX_HD Mat3 disp_grad(const float d1[3], const float d2[3], const float d3[3], const float* Dmi) {
    Mat3 H;
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++) H.m[3 * i + j] = d1[i] * Dmi[j] + d2[i] * Dmi[3 + j] + d3[i] * Dmi[6 + j];
    }
    return H;
}

// det(I + H) - 1 = tr H + i2(H) + det H
NFX_HD float det1p_minus1(const Mat3& H) {
    const float* h = H.m;
    const float t = h[0] + h[4] + h[8];
    const float i2 = (h[0] * h[4] - h[1] * h[3]) + (h[4] * h[8] - h[5] * h[7]) + (h[0] * h[8] - h[2] * h[6]);
    const float d = h[0] * (h[4] * h[8] - h[5] * h[7]) - h[1] * (h[3] * h[8] - h[5] * h[6]) +
                    h[2] * (h[3] * h[7] - h[4] * h[6]);
    return t + (i2 + d);
}

// E = B - I = H + H^T + H H^T for F = I + H, B = F F^T
NFX_HD Sym3 left_strain(const Mat3& H) {
    const float* h = H.m;
    Sym3 E;
    E.xx = 2.0f * h[0] + (h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    E.yy = 2.0f * h[4] + (h[3] * h[3] + h[4] * h[4] + h[5] * h[5]);
    E.zz = 2.0f * h[8] + (h[6] * h[6] + h[7] * h[7] + h[8] * h[8]);
    E.xy = (h[1] + h[3]) + (h[0] * h[3] + h[1] * h[4] + h[2] * h[5]);
    E.yz = (h[5] + h[7]) + (h[3] * h[6] + h[4] * h[7] + h[5] * h[8]);
    E.xz = (h[2] + h[6]) + (h[0] * h[6] + h[1] * h[7] + h[2] * h[8]);
    return E;
}

// Cauchy stress of the compressible Mooney-Rivlin law of tetra.cl:140-156 (and of
// InteractionFiniteStrainViscoplastic.cl:105-107), written in E = B - I and Jm1 = J - 1, as its
// deviatoric part and its pressure:
//   sigma = dev + kappa Jm1 I,
//   dev   = mu1 J^-5/3 dev(E) + mu2 J^-7/3 [(1 + e) dev(E) - dev(E^2)],   e = tr E.
// With B = I + E this equals the reference's
//   mu1 J^-5/3 (B - trB/3 I) + kappa (J-1) I + mu2 J^-7/3 (trB B - B^2 + (tr B^2 - trB^2)/3 I),
// whose mu2 term is traceless: trB B - B^2 + (tr B^2 - trB^2)/3 I = (1 + e) dev(E) - dev(E^2) +
// (e e/3 - tr(E^2)/3 + (tr(E^2) - e^2)/3) I and the bracket vanishes. Forming the deviator from
// deviatoric terms keeps it exact where the stress is mostly hydrostatic (under an indenter the
// pressure can be ten times the deviator): taking tr(sigma)/3 off a summed stress instead loses
// that ratio in FP32, and the viscoplastic flow, driven by the deviator every step, integrates
// the loss (measured: the 10^4-step curve error of the viscoplastic cell halves).
struct StressSplit {
    Sym3 dev;
    float p;  // pressure, tr(sigma)/3
};
NFX_HD StressSplit mr_stress_split(const Sym3& E, float Jm1, float mu1, float mu2, float kappa) {
    const float J = 1.0f + Jm1;
    const float c = rcbrt_(J);
    const float c2 = c * c;
    const float c5 = c2 * c2 * c;
    const float e = E.xx + E.yy + E.zz;
    const float e3 = e * (1.0f / 3.0f);
    Sym3 D;  // dev(E)
    D.xx = E.xx - e3;
    D.yy = E.yy - e3;
    D.zz = E.zz - e3;
    D.xy = E.xy;
    D.yz = E.yz;
    D.xz = E.xz;
    const float a1 = mu1 * c5;
    StressSplit r;
    r.p = kappa * Jm1;
    r.dev.xx = a1 * D.xx;
    r.dev.yy = a1 * D.yy;
    r.dev.zz = a1 * D.zz;
    r.dev.xy = a1 * D.xy;
    r.dev.yz = a1 * D.yz;
    r.dev.xz = a1 * D.xz;
    if (mu2 != 0.0f) {
        const float a2 = mu2 * c5 * c2;
        // E^2 (symmetric) and its trace / 3
        const float q_xx = E.xx * E.xx + E.xy * E.xy + E.xz * E.xz;
        const float q_yy = E.xy * E.xy + E.yy * E.yy + E.yz * E.yz;
        const float q_zz = E.xz * E.xz + E.yz * E.yz + E.zz * E.zz;
        const float q_xy = E.xx * E.xy + E.xy * E.yy + E.xz * E.yz;
        const float q_yz = E.xy * E.xz + E.yy * E.yz + E.yz * E.zz;
        const float q_xz = E.xx * E.xz + E.xy * E.yz + E.xz * E.zz;
        const float q3 = (q_xx + q_yy + q_zz) * (1.0f / 3.0f);
        const float k = 1.0f + e;
        r.dev.xx += a2 * (k * D.xx - (q_xx - q3));
        r.dev.yy += a2 * (k * D.yy - (q_yy - q3));
        r.dev.zz += a2 * (k * D.zz - (q_zz - q3));
        r.dev.xy += a2 * (k * D.xy - q_xy);
        r.dev.yz += a2 * (k * D.yz - q_yz);
        r.dev.xz += a2 * (k * D.xz - q_xz);
    }
    return r;
}

// The full Cauchy stress dev + p I.
NFX_HD Sym3 mr_stress(const Sym3& E, float Jm1, float mu1, float mu2, float kappa) {
    const StressSplit r = mr_stress_split(E, Jm1, mu1, mu2, kappa);
    Sym3 s = r.dev;
    s.xx += r.p;
    s.yy += r.p;
    s.zz += r.p;
    return s;
}

// adj(F) = det(F) F^-1 for F = I + H (cofactor transpose).
NFX_HD Mat3 adj_1p(const Mat3& H) {
    const float a = 1.0f + H.m[0], b = H.m[1], c = H.m[2];
    const float d = H.m[3], e = 1.0f + H.m[4], f = H.m[5];
    const float g = H.m[6], h = H.m[7], i = 1.0f + H.m[8];
    Mat3 A;
    A.m[0] = e * i - f * h;
    A.m[1] = c * h - b * i;
    A.m[2] = b * f - c * e;
    A.m[3] = f * g - d * i;
    A.m[4] = a * i - c * g;
    A.m[5] = c * d - a * f;
    A.m[6] = d * h - e * g;
    A.m[7] = b * g - a * h;
    A.m[8] = a * e - b * d;
    return A;
}

// Nodal forces from a Cauchy stress, tetra.cl:159-168: rows of -V0 * Dmi * A * sigma with
// A = adj(F) (= det(F) F^-1) give f1, f2, f3; f0 = -(f1 + f2 + f3). scale multiplies A
// (+1 for the elastic kernel, sign(det F) for the viscoplastic one whose current volume
// is |det Ds|/6, InteractionFiniteStrainViscoplastic.cl:126-141).
NFX_HD void forces_from_stress(const Mat3& A, const Sym3& s, const float* Dmi, float V0, float f[4][3]) {
    // P = A * sigma
    float P[9];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float a0 = A.m[3 * i], a1 = A.m[3 * i + 1], a2 = A.m[3 * i + 2];
        P[3 * i + 0] = a0 * s.xx + a1 * s.xy + a2 * s.xz;
        P[3 * i + 1] = a0 * s.xy + a1 * s.yy + a2 * s.yz;
        P[3 * i + 2] = a0 * s.xz + a1 * s.yz + a2 * s.zz;
    }
    const float w = -V0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float m0 = Dmi[3 * k] * w, m1 = Dmi[3 * k + 1] * w, m2 = Dmi[3 * k + 2] * w;
#pragma unroll
        for (int j = 0; j < 3; j++) f[k + 1][j] = m0 * P[j] + m1 * P[3 + j] + m2 * P[6 + j];
    }
#pragma unroll
    for (int j = 0; j < 3; j++) f[0][j] = -((f[1][j] + f[2][j]) + f[3][j]);
}

// The same forces from the stress split into its deviator and pressure (sigma = dev + p I).
NFX_HD void forces_from_split(const Mat3& A, const StressSplit& sp, const float* Dmi, float V0, float f[4][3]) {
    const Sym3& d = sp.dev;
    float P[9];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float a0 = A.m[3 * i], a1 = A.m[3 * i + 1], a2 = A.m[3 * i + 2];
        P[3 * i + 0] = a0 * (d.xx + sp.p) + a1 * d.xy + a2 * d.xz;
        P[3 * i + 1] = a0 * d.xy + a1 * (d.yy + sp.p) + a2 * d.yz;
        P[3 * i + 2] = a0 * d.xz + a1 * d.yz + a2 * (d.zz + sp.p);
    }
    const float w = -V0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float m0 = Dmi[3 * k] * w, m1 = Dmi[3 * k + 1] * w, m2 = Dmi[3 * k + 2] * w;
#pragma unroll
        for (int j = 0; j < 3; j++) f[k + 1][j] = m0 * P[j] + m1 * P[3 + j] + m2 * P[6 + j];
    }
#pragma unroll
    for (int j = 0; j < 3; j++) f[0][j] = -((f[1][j] + f[2][j]) + f[3][j]);
}

// Elastic Mooney-Rivlin / Neo-Hookean element, tetra.cl:115-168 (NH is mu2 = 0,
// nofluidx3d/interactions/Tetra.py:77-78). Returns det F - 1 (for inversion checks).
NFX_HD float mr_element(const float d1[3], const float d2[3], const float d3[3], const float* Dmi, float V0,
                        float mu1, float mu2, float kappa, float f[4][3]) {
    const Mat3 H = disp_grad(d1, d2, d3, Dmi);
    const float Jm1 = det1p_minus1(H);
    const Sym3 E = left_strain(H);
    const Sym3 s = mr_stress(E, Jm1, mu1, mu2, kappa);
    const Mat3 A = adj_1p(H);
    forces_from_stress(A, s, Dmi, V0, f);
    return Jm1;
}

// Saint-Venant-Kirchhoff variant of tetra.cl:94-114:
//   Force = -V0 mu Dm^-1 F^T (k' tr(B-I) I + (B-I)),   k' = nu/(1-2nu).
NFX_HD float svk_element(const float d1[3], const float d2[3], const float d3[3], const float* Dmi, float V0,
                         float mu, float kp, float f[4][3]) {
    const Mat3 H = disp_grad(d1, d2, d3, Dmi);
    const Sym3 E = left_strain(H);
    const float te = kp * (E.xx + E.yy + E.zz);
    const float S[9] = {E.xx + te, E.xy, E.xz, E.xy, E.yy + te, E.yz, E.xz, E.yz, E.zz + te};
    // Q = F^T S, F^T_ij = delta_ij + H_ji
    float Q[9];
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++)
            Q[3 * i + j] = S[3 * i + j] + (H.m[i] * S[j] + H.m[3 + i] * S[3 + j] + H.m[6 + i] * S[6 + j]);
    }
    const float w = -V0 * mu;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float m0 = Dmi[3 * k] * w, m1 = Dmi[3 * k + 1] * w, m2 = Dmi[3 * k + 2] * w;
#pragma unroll
        for (int j = 0; j < 3; j++) f[k + 1][j] = m0 * Q[j] + m1 * Q[3 + j] + m2 * Q[6 + j];
    }
#pragma unroll
    for (int j = 0; j < 3; j++) f[0][j] = -((f[1][j] + f[2][j]) + f[3][j]);
    return det1p_minus1(H);
}

// General 3x3 inverse by cofactors / det (matrix.cl:178-181).
NFX_HD Mat3 inv3(const Mat3& M) {
    const float* m = M.m;
    Mat3 A;
    A.m[0] = m[4] * m[8] - m[5] * m[7];
    A.m[1] = m[2] * m[7] - m[1] * m[8];
    A.m[2] = m[1] * m[5] - m[2] * m[4];
    A.m[3] = m[5] * m[6] - m[3] * m[8];
    A.m[4] = m[0] * m[8] - m[2] * m[6];
    A.m[5] = m[2] * m[3] - m[0] * m[5];
    A.m[6] = m[3] * m[7] - m[4] * m[6];
    A.m[7] = m[1] * m[6] - m[0] * m[7];
    A.m[8] = m[0] * m[4] - m[1] * m[3];
    const float det = m[0] * A.m[0] + m[1] * A.m[3] + m[2] * A.m[6];
    const float r = 1.0f / det;
#pragma unroll
    for (int k = 0; k < 9; k++) A.m[k] *= r;
    return A;
}

NFX_HD Mat3 mul3(const Mat3& a, const Mat3& b) {
    Mat3 r;
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    }
    return r;
}

NFX_HD Mat3 transpose3(const Mat3& a) {
    Mat3 r = {{a.m[0], a.m[3], a.m[6], a.m[1], a.m[4], a.m[7], a.m[2], a.m[5], a.m[8]}};
    return r;
}

// "Kellnberger" variant of tetra.cl:76-93: S = approximateRoot(B) (10 Newton steps of the
// orthogonal polar factor, :5-12), Force = -V0 mu Dm^-1 (I + (k'(tr S - 3) - 1) S^-1) F^T.
NFX_HD float svkk_element(const float d1[3], const float d2[3], const float d3[3], const float* Dmi, float V0,
                          float mu, float kp, float f[4][3]) {
    const Mat3 H = disp_grad(d1, d2, d3, Dmi);
    const Sym3 E = left_strain(H);
    const Mat3 B = {{1.0f + E.xx, E.xy, E.xz, E.xy, 1.0f + E.yy, E.yz, E.xz, E.yz, 1.0f + E.zz}};
    Mat3 X = B;
    for (int it = 0; it < 10; it++) {
        const Mat3 Xi = inv3(transpose3(X));
#pragma unroll
        for (int k = 0; k < 9; k++) X.m[k] = (X.m[k] + Xi.m[k]) * 0.5f;
    }
    const Mat3 S = mul3(transpose3(X), B);
    const Mat3 Si = inv3(S);
    const float sf = kp * ((S.m[0] + S.m[4] + S.m[8]) - 3.0f) - 1.0f;
    Mat3 inner;
#pragma unroll
    for (int k = 0; k < 9; k++) inner.m[k] = Si.m[k] * sf;
    inner.m[0] += 1.0f;
    inner.m[4] += 1.0f;
    inner.m[8] += 1.0f;
    // Q = inner * F^T
    float Q[9];
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++)
            Q[3 * i + j] = inner.m[3 * i + j] +
                           (inner.m[3 * i] * H.m[3 * j] + inner.m[3 * i + 1] * H.m[3 * j + 1] +
                            inner.m[3 * i + 2] * H.m[3 * j + 2]);
    }
    const float w = -V0 * mu;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float m0 = Dmi[3 * k] * w, m1 = Dmi[3 * k + 1] * w, m2 = Dmi[3 * k + 2] * w;
#pragma unroll
        for (int j = 0; j < 3; j++) f[k + 1][j] = m0 * Q[j] + m1 * Q[3 + j] + m2 * Q[6 + j];
    }
#pragma unroll
    for (int j = 0; j < 3; j++) f[0][j] = -((f[1][j] + f[2][j]) + f[3][j]);
    return det1p_minus1(H);
}

// Parameters of the viscoplastic law (InteractionFiniteStrainViscoplastic.cl:1, :105-156).
struct VPParams {
    float mu1, mu2, kappa, flow_exp, yield, flow_rate, hard_thr, hard_exp;
};

// Multiplicative finite-strain viscoplastic element,
// InteractionFiniteStrainViscoplastic.cl:30-206. The plastic deformation tensor is carried as
// its deviation from the identity, P = Fp - I, so that FP32 resolves the small per-step
// increments Fp += Fe^-1 Dp F (:171-206). Mathematically identical forms with fewer operations:
//   Fe - I = F Fp^-1 - I = (F - Fp) Fp^-1 = (H - P) adj(I + P) / det(I + P)      (:59-79)
//   Fe^-1 Dp F = Fp F^-1 Dp F = (I + P) M,   M = adj(F) Dp F / det F               (:171-195)
// Be = Fe Fe^T (:82-84), J = sqrt(det Be) = |det Fe| (:87), sigma of the Mooney-Rivlin law
// (:105-107), nodal forces one third of the adjacent face tractions (:110-141), which for a
// linear tetrahedron equal -|V| sigma grad N_i, i.e. rows of -V0 sign(det F) Dm^-1 adj(F) sigma.
// Reads P (9); writes its increment dP (9) and the plastic strain rate, which the caller adds
// to its stored state; writes von Mises and pressure.
NFX_HD void vp_element(const float d1[3], const float d2[3], const float d3[3], const float* Dmi, float V0,
                       const VPParams& par, const float Pp[9], float eps, float dP[9], float& rate_out,
                       float f[4][3], float& vm_out, float& p_out, float& Jm1_out) {
    const Mat3 H = disp_grad(d1, d2, d3, Dmi);
    Mat3 Pm;
#pragma unroll
    for (int k = 0; k < 9; k++) Pm.m[k] = Pp[k];
    const Mat3 adjFp = adj_1p(Pm);
    // det(I + P) by expansion along the first row of the adjugate already formed
    const float rdet = fdiv_(1.0f, (1.0f + Pm.m[0]) * adjFp.m[0] + Pm.m[1] * adjFp.m[3] + Pm.m[2] * adjFp.m[6]);
    Mat3 D;
#pragma unroll
    for (int k = 0; k < 9; k++) D.m[k] = H.m[k] - Pm.m[k];
    Mat3 G = mul3(D, adjFp);
#pragma unroll
    for (int k = 0; k < 9; k++) G.m[k] *= rdet;
    // elastic left strain and volume change
    const Sym3 Ee = left_strain(G);
    const float JeM1 = det1p_minus1(G);  // det Fe - 1
    const float Je = 1.0f + JeM1;
    const float JabsM1 = Je >= 0.0f ? JeM1 : (-Je - 1.0f);  // J = sqrt(det Be) = |det Fe|
    const StressSplit sp = mr_stress_split(Ee, JabsM1, par.mu1, par.mu2, par.kappa);
    const Sym3& s = sp.dev;  // the shear components of sigma and its deviator coincide
    // forces
    const float JFm1 = det1p_minus1(H);
    const Mat3 A = adj_1p(H);
    const float sgn = (1.0f + JFm1) >= 0.0f ? 1.0f : -1.0f;
    forces_from_split(A, sp, Dmi, (V0 >= 0.0f ? V0 : -V0) * sgn, f);
    Jm1_out = JFm1;
    // flow rule (:144-169), driven by the deviatoric stress formed directly
    const float t3 = sp.p;
    const float dxx = sp.dev.xx, dyy = sp.dev.yy, dzz = sp.dev.zz;
    const float vm = sqrt_(1.5f * ((dxx * dxx + dyy * dyy + dzz * dzz) +
                                   2.0f * (s.xy * s.xy + s.yz * s.yz + s.xz * s.xz)));
    const float sigma0 = par.yield * (par.hard_exp == 0.0f ? 1.0f : pow_(1.0f + eps / par.hard_thr, par.hard_exp));
    vm_out = vm;
    p_out = t3;
    // linear flow law: rate / vm is the constant flow_rate / sigma0 (one division)
    float rate, kv;
    if (par.flow_exp == 1.0f) {
        const float q = fdiv_(par.flow_rate, sigma0);
        rate = q * vm;
        kv = 1.5f * q;
    } else {
        rate = par.flow_rate * pow_(fdiv_(vm, sigma0), par.flow_exp);
        kv = vm != 0.0f ? fdiv_(rate * 1.5f, vm) : 0.0f;
    }
    rate_out = rate;
#pragma unroll
    for (int q = 0; q < 9; q++) dP[q] = 0.0f;
    if (vm != 0.0f) {
        const float rJ = fdiv_(1.0f, 1.0f + JFm1);
        const float k = kv * rJ;  // 1/det F folded into the scale of Dp
        const float Dp[9] = {dxx * k, s.xy * k, s.xz * k, s.xy * k, dyy * k, s.yz * k, s.xz * k, s.yz * k, dzz * k};
        // T = adj(F) Dp / det F (the 1/det F inside k), then M = T (I + H)
        float T[9];
#pragma unroll
        for (int i = 0; i < 3; i++) {
#pragma unroll
            for (int j = 0; j < 3; j++)
                T[3 * i + j] = A.m[3 * i] * Dp[j] + A.m[3 * i + 1] * Dp[3 + j] + A.m[3 * i + 2] * Dp[6 + j];
        }
        float M[9];
#pragma unroll
        for (int i = 0; i < 3; i++) {
#pragma unroll
            for (int j = 0; j < 3; j++)
                M[3 * i + j] = T[3 * i + j] + (T[3 * i] * H.m[j] + T[3 * i + 1] * H.m[3 + j] +
                                               T[3 * i + 2] * H.m[6 + j]);
        }
        // dP = (I + P) M
#pragma unroll
        for (int i = 0; i < 3; i++) {
#pragma unroll
            for (int j = 0; j < 3; j++)
                dP[3 * i + j] = M[3 * i + j] + (Pm.m[3 * i] * M[j] + Pm.m[3 * i + 1] * M[3 + j] +
                                                Pm.m[3 * i + 2] * M[6 + j]);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Double-float (hi + lo) helpers for the node state (displacement and velocity), so that
// per-step increments of 1e-4 against values of O(1) accumulate without FP32 drift.
// TwoSum (Knuth) is exact for any inputs; a quick renormalisation keeps |lo| <= ulp(hi)/2.
// ---------------------------------------------------------------------------------------
NFX_HD void df_add(float& hi, float& lo, float a) {
    const float s = hi + a;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (a - bb);
    const float l = lo + err;
    const float h2 = s + l;
    lo = l - (h2 - s);
    hi = h2;
}

}  // namespace nfx
