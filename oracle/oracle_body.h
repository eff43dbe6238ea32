/*
 * CPU restatement of noFluidX3D's explicit tetra-mesh step (ORACLE: test infrastructure only).
 *
 * This body is included twice by nfx_oracle.c, once with `real` = double (suffix _f64, the
 * precision the reference ships in, nofluidx3d/kernels/typedefs.h:1-7) and once with
 * `real` = float (suffix _f32). Every function restates one reference kernel or host routine
 * and cites it. Buffers use the reference's layouts:
 *   points / force / velocity / fold : SoA, component d of node i at [d*np + i]
 *                                      (nofluidx3d/Simulation.py:82-88)
 *   tets                              : SoA u32, corner k of tet t at [k*nt + t] (Simulation.py:85-87)
 *   edge                              : SoA, entry k of tet t at [k*nt + t], k = 3*vector + component
 *                                      (nofluidx3d/interactions/Tetra.py:53-55)
 *   Fp (viscoplastic)                 : SoA, entry k of tet t at [k*nt + t], row-major 3x3
 *                                      (nofluidx3d/Interactions.py:279-281)
 * Work-items are executed in index order, so the reference's CAS atomics
 * (nofluidx3d/kernels/atomicAdd.cl:1-11) become plain additions in tet order.
 * Nothing in the product links this file; it is only the checker.
 */
#define NAME_(a, b) a##b
#define NAME2(a, b) NAME_(a, b)
#define NM(n) NAME2(n, SFX)

#define V3 NM(ora_v3)
#define M3 NM(ora_m3)

typedef struct { real x, y, z; } V3;
typedef struct { real m11, m12, m13, m21, m22, m23, m31, m32, m33; } M3;

/* ---- 3-vector helpers: OpenCL built-ins dot/cross/length/normalize/max ---- */
static inline V3 NM(mk3)(real x, real y, real z) { V3 r = {x, y, z}; return r; }
static inline V3 NM(vadd)(V3 a, V3 b) { return NM(mk3)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 NM(vsub)(V3 a, V3 b) { return NM(mk3)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 NM(vneg)(V3 a) { return NM(mk3)(-a.x, -a.y, -a.z); }
static inline V3 NM(vscale)(V3 a, real s) { return NM(mk3)(a.x * s, a.y * s, a.z * s); }
static inline V3 NM(vdiv)(V3 a, real s) { return NM(mk3)(a.x / s, a.y / s, a.z / s); }
static inline real NM(vdot)(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 NM(vcross)(V3 a, V3 b) {
    return NM(mk3)(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline real NM(vlen)(V3 a) { return SQRT(NM(vdot)(a, a)); }
static inline V3 NM(vnormalize)(V3 a) { return NM(vdiv)(a, NM(vlen)(a)); }

/* ---- 3x3 helpers, nofluidx3d/kernels/matrix.cl:118-218 (Double3x3, 1-based rows/columns) ---- */
static inline M3 NM(from_cols)(V3 c1, V3 c2, V3 c3) {
    M3 m = {c1.x, c2.x, c3.x, c1.y, c2.y, c3.y, c1.z, c2.z, c3.z};
    return m;
}
static inline M3 NM(from_rows)(V3 r1, V3 r2, V3 r3) {
    M3 m = {r1.x, r1.y, r1.z, r2.x, r2.y, r2.z, r3.x, r3.y, r3.z};
    return m;
}
static inline V3 NM(row)(M3 m, int i) {
    return i == 1 ? NM(mk3)(m.m11, m.m12, m.m13) : i == 2 ? NM(mk3)(m.m21, m.m22, m.m23)
                                                          : NM(mk3)(m.m31, m.m32, m.m33);
}
static inline V3 NM(col)(M3 m, int j) {
    return j == 1 ? NM(mk3)(m.m11, m.m21, m.m31) : j == 2 ? NM(mk3)(m.m12, m.m22, m.m32)
                                                          : NM(mk3)(m.m13, m.m23, m.m33);
}
static inline real NM(tr)(M3 m) { return m.m11 + m.m22 + m.m33; }
/* det = col1 . (col2 x col3)  (matrix.cl:166-168) */
static inline real NM(det)(M3 m) {
    return NM(vdot)(NM(col)(m, 1), NM(vcross)(NM(col)(m, 2), NM(col)(m, 3)));
}
static inline M3 NM(transpose)(M3 m) {
    M3 t = {m.m11, m.m21, m.m31, m.m12, m.m22, m.m32, m.m13, m.m23, m.m33};
    return t;
}
static inline M3 NM(mscale)(M3 m, real s) {
    M3 r = {m.m11 * s, m.m12 * s, m.m13 * s, m.m21 * s, m.m22 * s,
            m.m23 * s, m.m31 * s, m.m32 * s, m.m33 * s};
    return r;
}
/* devide(m, s) = multiply(m, 1/s)  (matrix.cl:216-218) */
static inline M3 NM(mdivs)(M3 m, real s) { return NM(mscale)(m, (real)1 / s); }
/* invert = rows of cofactor crosses / det  (matrix.cl:178-181) */
static inline M3 NM(invert)(M3 m) {
    V3 c1 = NM(col)(m, 1), c2 = NM(col)(m, 2), c3 = NM(col)(m, 3);
    return NM(mdivs)(NM(from_rows)(NM(vcross)(c2, c3), NM(vcross)(c3, c1), NM(vcross)(c1, c2)),
                     NM(det)(m));
}
static inline M3 NM(madd)(M3 a, M3 b) {
    return NM(from_rows)(NM(vadd)(NM(row)(a, 1), NM(row)(b, 1)), NM(vadd)(NM(row)(a, 2), NM(row)(b, 2)),
                         NM(vadd)(NM(row)(a, 3), NM(row)(b, 3)));
}
static inline M3 NM(msub)(M3 a, M3 b) {
    return NM(from_rows)(NM(vsub)(NM(row)(a, 1), NM(row)(b, 1)), NM(vsub)(NM(row)(a, 2), NM(row)(b, 2)),
                         NM(vsub)(NM(row)(a, 3), NM(row)(b, 3)));
}
/* (matrix.cl:195-201) entry ij = row_i(a) . col_j(b) */
static inline M3 NM(mmul)(M3 a, M3 b) {
    M3 r;
    V3 a1 = NM(row)(a, 1), a2 = NM(row)(a, 2), a3 = NM(row)(a, 3);
    V3 b1 = NM(col)(b, 1), b2 = NM(col)(b, 2), b3 = NM(col)(b, 3);
    r.m11 = NM(vdot)(a1, b1); r.m12 = NM(vdot)(a1, b2); r.m13 = NM(vdot)(a1, b3);
    r.m21 = NM(vdot)(a2, b1); r.m22 = NM(vdot)(a2, b2); r.m23 = NM(vdot)(a2, b3);
    r.m31 = NM(vdot)(a3, b1); r.m32 = NM(vdot)(a3, b2); r.m33 = NM(vdot)(a3, b3);
    return r;
}
static inline M3 NM(unit)(void) { M3 u = {1, 0, 0, 0, 1, 0, 0, 0, 1}; return u; }

static inline V3 NM(load3)(const real* a, long n, long i) { return NM(mk3)(a[i], a[n + i], a[2 * n + i]); }
static inline void NM(add3)(real* a, long n, long i, V3 v) {
    a[i] += v.x;
    a[n + i] += v.y;
    a[2 * n + i] += v.z;
}

/* Newton iteration for the orthogonal polar factor, nofluidx3d/kernels/Interactions/tetra.cl:5-12:
 * X <- (X + X^-T)/2 ten times, returns X^T * initial. */
static M3 NM(approx_root)(M3 initial) {
    M3 it = initial;
    for (int i = 0; i < 10; i++) it = NM(mdivs)(NM(madd)(it, NM(invert)(NM(transpose)(it))), (real)2);
    return NM(mmul)(NM(transpose)(it), initial);
}

/* Per-tetra hyperelastic forces, nofluidx3d/kernels/Interactions/tetra.cl:14-182.
 * model: 0 = Mooney-Rivlin / Neo-Hookean (:115-163), 1 = Saint-Venant-Kirchhoff (:94-114),
 *        2 = SVK "Kellnberger" with polar decomposition (:76-93).
 * Material constants are those KernelBuilder bakes in (nofluidx3d/interactions/Tetra.py:68-79). */
static void NM(tet_force_one)(long t, long np, long nt, const real* points, const unsigned* tets,
                              const real* edge, const real* vol, int model, real E, real nu, real mr,
                              V3* fout) {
    const unsigned i0 = tets[t], i1 = tets[nt + t], i2 = tets[2 * nt + t], i3 = tets[3 * nt + t];
    const V3 p0 = NM(load3)(points, np, i0), p1 = NM(load3)(points, np, i1);
    const V3 p2 = NM(load3)(points, np, i2), p3 = NM(load3)(points, np, i3);
    const V3 r1 = NM(vsub)(p1, p0), r2 = NM(vsub)(p2, p0), r3 = NM(vsub)(p3, p0);
    const M3 rT = NM(from_cols)(r1, r2, r3);
    const V3 R1 = NM(mk3)(edge[t], edge[nt + t], edge[2 * nt + t]);
    const V3 R2 = NM(mk3)(edge[3 * nt + t], edge[4 * nt + t], edge[5 * nt + t]);
    const V3 R3 = NM(mk3)(edge[6 * nt + t], edge[7 * nt + t], edge[8 * nt + t]);
    const real V0 = vol[t];
    const M3 J = NM(from_cols)(R1, R2, R3);
    const M3 invJ = NM(invert)(J);                 /* :53 */
    const M3 F = NM(mmul)(rT, invJ);               /* :63 */
    const M3 FT = NM(transpose)(F);
    const M3 B = NM(mmul)(F, FT);                  /* :68 */
    const M3 uT = NM(unit)();
    M3 Force;
    if (model == 2) {                              /* :76-93 */
        const real kappa = nu / (1 - 2 * nu);
        const real mu = E / (2 * (1 + nu));
        const M3 S = NM(approx_root)(B);
        const M3 invS = NM(invert)(S);
        const real sf = kappa * (NM(tr)(S) - 3) - 1;
        const M3 inner = NM(madd)(uT, NM(mscale)(invS, sf));
        Force = NM(mscale)(NM(mmul)(NM(mmul)(invJ, inner), FT), -V0 * mu);
    } else if (model == 1) {                       /* :94-114 */
        const real kappa = nu / (1 - 2 * nu);
        const real mu = E / (2 * (1 + nu));
        const M3 BP = NM(msub)(B, uT);
        const M3 H = NM(mmul)(invJ, FT);
        const M3 term1 = NM(mscale)(H, kappa * NM(tr)(BP));
        const M3 term2 = NM(mmul)(H, BP);
        Force = NM(mscale)(NM(madd)(term1, term2), -V0 * mu);
    } else {                                       /* :115-163 */
        const real mu = E / (2 * (1 + nu));
        const real mu1 = mr * mu;
        const real mu2 = (1 - mr) * mu;
        const real kappa = E / (3 * (1 - 2 * nu));
        const M3 Bsq = NM(mmul)(B, B);
        const real trB = NM(tr)(B);
        const real trBsq = NM(tr)(Bsq);
        const real Jr = NM(det)(rT) / (6 * V0);    /* :132 */
        const real dUdI1 = mu1 / POW(Jr, 5 / (real)3);
        const real dUdK = mu2 / POW(Jr, 7 / (real)3);
        const real dUdJ = kappa * (Jr - 1);
        const real dI1dJ = -trB / 3;
        const M3 term1 = NM(mscale)(B, dUdI1);
        const M3 term2 = NM(mscale)(uT, dUdJ + dI1dJ * dUdI1);
        const M3 inner1 = NM(msub)(NM(mscale)(B, trB), Bsq);
        const M3 inner2 = NM(mscale)(uT, (trBsq - trB * trB) / 3);
        const M3 term3 = NM(mscale)(NM(madd)(inner1, inner2), dUdK);
        const M3 sigma = NM(madd)(NM(madd)(term1, term2), term3);
        const M3 helper = NM(mmul)(NM(invert)(rT), sigma);   /* :159 */
        Force = NM(mscale)(helper, -V0 * Jr);                 /* :162 */
    }
    fout[1] = NM(row)(Force, 1);
    fout[2] = NM(row)(Force, 2);
    fout[3] = NM(row)(Force, 3);
    fout[0] = NM(vneg)(NM(vadd)(NM(vadd)(fout[1], fout[2]), fout[3]));  /* :168 */
    (void)i0; (void)i1; (void)i2; (void)i3;
}

void NM(ora_tet_force)(long np, long nt, const real* points, const unsigned* tets, const real* edge,
                       const real* vol, int model, real E, real nu, real mr, real* force) {
    for (long t = 0; t < nt; t++) {
        V3 f[4];
        NM(tet_force_one)(t, np, nt, points, tets, edge, vol, model, E, nu, mr, f);
        for (int k = 0; k < 4; k++) NM(add3)(force, np, tets[k * nt + t], f[k]);  /* :170-181 */
    }
}

/* Multiplicative finite-strain viscoplasticity with a Mooney-Rivlin elastic law,
 * nofluidx3d/kernels/InteractionFiniteStrainViscoplastic.cl:1-220. The base node is corner 3
 * (the kernel's "point 4", :18-22), so edge must hold R_i = P_i - P_3. Material parameters are
 * uniform scalars, as the only wrapper fills them (nofluidx3d/Interactions.py:270-281).
 * par = {mu1, mu2, kappa, flowExponent, yieldStress, plasticFlowRate, hardeningThreshhold,
 *        hardeningExponent}. accStrain, Fp, vonMises, pressure are updated in place. */
static void NM(vp_one)(long t, long np, long nt, const real* points, const unsigned* tets,
                       const real* edge, const real* par, real* acc, real* Fp, real* vonMises,
                       real* pressure, V3* fout) {
    const real mu1 = par[0], mu2 = par[1], kap = par[2], mexp = par[3], Y = par[4], rate0 = par[5];
    const real eps0 = par[6], nexp = par[7];
    const V3 p1 = NM(load3)(points, np, tets[t]), p2 = NM(load3)(points, np, tets[nt + t]);
    const V3 p3 = NM(load3)(points, np, tets[2 * nt + t]), p4 = NM(load3)(points, np, tets[3 * nt + t]);
    const V3 r1 = NM(vsub)(p1, p4), r2 = NM(vsub)(p2, p4), r3 = NM(vsub)(p3, p4);
    const V3 R1 = NM(mk3)(edge[t], edge[nt + t], edge[2 * nt + t]);
    const V3 R2 = NM(mk3)(edge[3 * nt + t], edge[4 * nt + t], edge[5 * nt + t]);
    const V3 R3 = NM(mk3)(edge[6 * nt + t], edge[7 * nt + t], edge[8 * nt + t]);
    const V3 u1 = NM(vsub)(r1, R1), u2 = NM(vsub)(r2, R2), u3 = NM(vsub)(r3, R3);  /* :32-34 */
    const real divisor = NM(vdot)(NM(vcross)(R1, R2), R3);
    const V3 iJ1 = NM(vdiv)(NM(vcross)(R2, R3), divisor);
    const V3 iJ2 = NM(vdiv)(NM(vcross)(R3, R1), divisor);
    const V3 iJ3 = NM(vdiv)(NM(vcross)(R1, R2), divisor);
    /* :47-55  F_k = du_k/dR + e_k */
    const V3 d1 = NM(vadd)(NM(vadd)(NM(vscale)(iJ1, u1.x), NM(vscale)(iJ2, u2.x)), NM(vscale)(iJ3, u3.x));
    const V3 d2 = NM(vadd)(NM(vadd)(NM(vscale)(iJ1, u1.y), NM(vscale)(iJ2, u2.y)), NM(vscale)(iJ3, u3.y));
    const V3 d3 = NM(vadd)(NM(vadd)(NM(vscale)(iJ1, u1.z), NM(vscale)(iJ2, u2.z)), NM(vscale)(iJ3, u3.z));
    const V3 F1 = NM(vadd)(d1, NM(mk3)(1, 0, 0)), F2 = NM(vadd)(d2, NM(mk3)(0, 1, 0));
    const V3 F3 = NM(vadd)(d3, NM(mk3)(0, 0, 1));
    /* :59-79  Fe = F * Fp^-1 with the adjugate inverse */
    real a = Fp[0 * nt + t], b = Fp[1 * nt + t], c = Fp[2 * nt + t], d = Fp[3 * nt + t];
    real e = Fp[4 * nt + t], f = Fp[5 * nt + t], g = Fp[6 * nt + t], h = Fp[7 * nt + t];
    real i = Fp[8 * nt + t];
    const real detFp = NM(vdot)(NM(vcross)(NM(mk3)(a, b, c), NM(mk3)(d, e, f)), NM(mk3)(g, h, i));
    const real ip = (real)1. / detFp;
    const V3 iF1 = NM(vscale)(NM(mk3)(e * i - f * h, c * h - b * i, b * f - c * e), ip);
    const V3 iF2 = NM(vscale)(NM(mk3)(f * g - d * i, a * i - c * g, c * d - a * f), ip);
    const V3 iF3 = NM(vscale)(NM(mk3)(d * h - e * g, b * g - a * h, a * e - b * d), ip);
#define ROWMUL(Fr) NM(mk3)(Fr.x * iF1.x + Fr.y * iF2.x + Fr.z * iF3.x, \
                           Fr.x * iF1.y + Fr.y * iF2.y + Fr.z * iF3.y, \
                           Fr.x * iF1.z + Fr.y * iF2.z + Fr.z * iF3.z)
    const V3 Fe1 = ROWMUL(F1), Fe2 = ROWMUL(F2), Fe3 = ROWMUL(F3);
#undef ROWMUL
    /* :82-96  Be = Fe Fe^T, J = sqrt(det Be), Be^2, traces */
    const V3 B1 = NM(mk3)(NM(vdot)(Fe1, Fe1), NM(vdot)(Fe1, Fe2), NM(vdot)(Fe1, Fe3));
    const V3 B2 = NM(mk3)(NM(vdot)(Fe2, Fe1), NM(vdot)(Fe2, Fe2), NM(vdot)(Fe2, Fe3));
    const V3 B3 = NM(mk3)(NM(vdot)(Fe3, Fe1), NM(vdot)(Fe3, Fe2), NM(vdot)(Fe3, Fe3));
    const real J = SQRT(NM(vdot)(NM(vcross)(B1, B2), B3));
#define SQROW(Br) NM(mk3)(Br.x * B1.x + Br.y * B2.x + Br.z * B3.x, Br.x * B1.y + Br.y * B2.y + Br.z * B3.y, \
                          Br.x * B1.z + Br.y * B2.z + Br.z * B3.z)
    const V3 S1 = SQROW(B1), S2 = SQROW(B2), S3 = SQROW(B3);
#undef SQROW
    const real trB = B1.x + B2.y + B3.z;
    const real trBsq = S1.x + S2.y + S3.z;
    const V3 E1 = NM(mk3)(1, 0, 0), E2 = NM(mk3)(0, 1, 0), E3 = NM(mk3)(0, 0, 1);
    /* :105-107  Cauchy stress of the compressible Mooney-Rivlin law */
    const real c53 = POW(J, (real)(-5.0 / 3.0)), c73 = POW(J, (real)(-7.0 / 3.0));
#define SIGROW(Br, Sr, Er)                                                                              \
    NM(vadd)(NM(vadd)(NM(vscale)(NM(vsub)(Br, NM(vscale)(Er, (real)(1. / 3.) * trB)), mu1 * c53),          \
                      NM(vscale)(Er, kap * (J - 1))),                                                   \
             NM(vscale)(NM(vadd)(NM(vsub)(NM(vsub)(NM(vscale)(Br, trB), NM(vscale)(Er, (real)(1.0 / 3.0) * trB * trB)), Sr), \
                                 NM(vscale)(Er, (real)(1.0 / 3.0) * trBsq)),                             \
                        mu2 * c73))
    const V3 sg1 = SIGROW(B1, S1, E1), sg2 = SIGROW(B2, S2, E2), sg3 = SIGROW(B3, S3, E3);
#undef SIGROW
    /* :110-141  outward unit normals, face areas, one third of the traction of adjacent faces */
    V3 n1 = NM(vcross)(r2, r3), n2 = NM(vcross)(r3, r1), n3 = NM(vcross)(r1, r2);
    V3 n4 = NM(vcross)(NM(vsub)(r3, r1), NM(vsub)(r3, r2));
    n1 = NM(vdiv)(n1, NM(vlen)(n1));
    n2 = NM(vdiv)(n2, NM(vlen)(n2));
    n3 = NM(vdiv)(n3, NM(vlen)(n3));
    n4 = NM(vdiv)(n4, NM(vlen)(n4));
    if (NM(vdot)(n1, NM(vneg)(r1)) < 0) n1 = NM(vscale)(n1, (real)-1);
    if (NM(vdot)(n2, NM(vneg)(r2)) < 0) n2 = NM(vscale)(n2, (real)-1);
    if (NM(vdot)(n3, NM(vneg)(r3)) < 0) n3 = NM(vscale)(n3, (real)-1);
    if (NM(vdot)(n4, r1) < 0) n4 = NM(vscale)(n4, (real)-1);
    const real A1 = (real)0.5 * NM(vlen)(NM(vcross)(r2, r3));
    const real A2 = (real)0.5 * NM(vlen)(NM(vcross)(r3, r1));
    const real A3 = (real)0.5 * NM(vlen)(NM(vcross)(r1, r2));
    const real A4 = (real)0.5 * NM(vlen)(NM(vcross)(NM(vsub)(r3, r1), NM(vsub)(r3, r2)));
#define TRAC(A, n) NM(vscale)(NM(mk3)(NM(vdot)(sg1, n), NM(vdot)(sg2, n), NM(vdot)(sg3, n)), A)
    const V3 fA1 = TRAC(A1, n1), fA2 = TRAC(A2, n2), fA3 = TRAC(A3, n3), fA4 = TRAC(A4, n4);
#undef TRAC
    const real m13 = (real)(-1.0 / 3.0);
    fout[0] = NM(vscale)(NM(vadd)(NM(vadd)(fA2, fA3), fA4), m13);
    fout[1] = NM(vscale)(NM(vadd)(NM(vadd)(fA3, fA4), fA1), m13);
    fout[2] = NM(vscale)(NM(vadd)(NM(vadd)(fA4, fA1), fA2), m13);
    fout[3] = NM(vscale)(NM(vadd)(NM(vadd)(fA1, fA2), fA3), m13);
    /* :144-156  von Mises stress, hardening, power-law plastic stretch rate */
    const real trS = sg1.x + sg2.y + sg3.z;
    const V3 ds1 = NM(vsub)(sg1, NM(vscale)(E1, trS / (real)3.0));
    const V3 ds2 = NM(vsub)(sg2, NM(vscale)(E2, trS / (real)3.0));
    const V3 ds3 = NM(vsub)(sg3, NM(vscale)(E3, trS / (real)3.0));
    const real vm = SQRT((real)(3. / 2.) * (NM(vdot)(ds1, ds1) + NM(vdot)(ds2, ds2) + NM(vdot)(ds3, ds3)));
    const real sigma0 = Y * POW((1 + acc[t] / eps0), nexp);
    vonMises[t] = vm;
    pressure[t] = trS / (real)3.0;
    const real rate = rate0 * POW(vm / sigma0, mexp);
    acc[t] += rate;
    /* :160-169  Dp = 3/2 rate dev(sigma)/sigma_vm */
    V3 Dp1, Dp2, Dp3;
    if (vm != 0) {
        Dp1 = NM(vdiv)(NM(vscale)(ds1, rate * (real)(3. / 2.)), vm);
        Dp2 = NM(vdiv)(NM(vscale)(ds2, rate * (real)(3. / 2.)), vm);
        Dp3 = NM(vdiv)(NM(vscale)(ds3, rate * (real)(3. / 2.)), vm);
    } else {
        Dp1 = Dp2 = Dp3 = NM(mk3)(0, 0, 0);
    }
    /* :171-206  Fp += Fe^-1 Dp F */
    a = Fe1.x; b = Fe1.y; c = Fe1.z; d = Fe2.x; e = Fe2.y; f = Fe2.z; g = Fe3.x; h = Fe3.y; i = Fe3.z;
    const real detFe = NM(vdot)(NM(vcross)(Fe1, Fe2), Fe3);
    const real ie = (real)1. / detFe;
    const V3 iE1 = NM(vscale)(NM(mk3)(e * i - f * h, c * h - b * i, b * f - c * e), ie);
    const V3 iE2 = NM(vscale)(NM(mk3)(f * g - d * i, a * i - c * g, c * d - a * f), ie);
    const V3 iE3 = NM(vscale)(NM(mk3)(d * h - e * g, b * g - a * h, a * e - b * d), ie);
#define TMP(r) NM(mk3)(r.x * Dp1.x + r.y * Dp2.x + r.z * Dp3.x, r.x * Dp1.y + r.y * Dp2.y + r.z * Dp3.y, \
                       r.x * Dp1.z + r.y * Dp2.z + r.z * Dp3.z)
    const V3 t1 = TMP(iE1), t2 = TMP(iE2), t3 = TMP(iE3);
#undef TMP
#define DOTF(r) NM(mk3)(r.x * F1.x + r.y * F2.x + r.z * F3.x, r.x * F1.y + r.y * F2.y + r.z * F3.y, \
                        r.x * F1.z + r.y * F2.z + r.z * F3.z)
    const V3 q1 = DOTF(t1), q2 = DOTF(t2), q3 = DOTF(t3);
#undef DOTF
    Fp[0 * nt + t] += q1.x; Fp[1 * nt + t] += q1.y; Fp[2 * nt + t] += q1.z;
    Fp[3 * nt + t] += q2.x; Fp[4 * nt + t] += q2.y; Fp[5 * nt + t] += q2.z;
    Fp[6 * nt + t] += q3.x; Fp[7 * nt + t] += q3.y; Fp[8 * nt + t] += q3.z;
}

void NM(ora_vp_force)(long np, long nt, const real* points, const unsigned* tets, const real* edge,
                      const real* par, real* acc, real* Fp, real* vonMises, real* pressure,
                      real* force) {
    for (long t = 0; t < nt; t++) {
        V3 f[4];
        NM(vp_one)(t, np, nt, points, tets, edge, par, acc, Fp, vonMises, pressure, f);
        for (int k = 0; k < 4; k++) NM(add3)(force, np, tets[k * nt + t], f[k]);  /* :209-220 */
    }
}

/* Substrate below the cell, nofluidx3d/kernels/Interactions/Substrate.cl:1-7 */
static inline void NM(substrate_node)(long i, long np, const real* points, real wall, real k, real* force) {
    real dis = FMAX(wall - points[np + i], (real)0.);
    force[np + i] += k * dis;
}
/* Flat indenter from above, nofluidx3d/kernels/Interactions/Plane.cl:1-7 */
static inline void NM(plane_node)(long i, long np, const real* points, real wall, real k, real* force) {
    real dis = FMAX(points[np + i] - wall, (real)0.);
    force[np + i] += -k * dis;
}
/* Spherical indenter centred at (0, spherePos, 0), nofluidx3d/kernels/Interactions/Sphere.cl:1-17 */
static inline void NM(sphere_node)(long i, long np, const real* points, real radius, real spos, real k,
                                   real* force) {
    const V3 pos = NM(load3)(points, np, i);
    const V3 r = NM(vsub)(pos, NM(mk3)(0, spos, 0));
    const V3 n = NM(vnormalize)(r);
    const real dis = FMAX(radius - NM(vlen)(r), (real)0.);
    const V3 fv = NM(vscale)(n, k * dis);
    NM(add3)(force, np, i, fv);
}
/* Damped velocity Verlet with unit mass and dt = 1, nofluidx3d/kernels/Interactions/VelocityVerlet.cl:1-36.
 * The reference hard-codes xi = 0.005 (:11); here it is the parameter xi. */
static inline void NM(vv_node)(long i, long np, real* points, real* vel, real* force, real* fold, real xi,
                               int fix_top_bottom) {
    V3 x = NM(load3)(points, np, i), v = NM(load3)(vel, np, i);
    V3 f = NM(load3)(force, np, i), fo = NM(load3)(fold, np, i);
    const real dm = 1 - (real)0.5 * xi, dp = 1 + (real)0.5 * xi;
    v = NM(vdiv)(NM(vadd)(NM(vscale)(v, dm), NM(vscale)(NM(vadd)(f, fo), (real)0.5)), dp);
    x = NM(vadd)(NM(vadd)(x, NM(vscale)(v, dm)), NM(vscale)(f, (real)0.5));
    fo = f;
    if (fix_top_bottom && (i == 3 || i == 4)) { x.x = 0; x.z = 0; }  /* :17-22 */
    points[i] = x.x; points[np + i] = x.y; points[2 * np + i] = x.z;
    vel[i] = v.x; vel[np + i] = v.y; vel[2 * np + i] = v.z;
    fold[i] = fo.x; fold[np + i] = fo.y; fold[2 * np + i] = fo.z;
    force[i] = 0; force[np + i] = 0; force[2 * np + i] = 0;
}

/* Lumped-mass damped velocity Verlet, nofluidx3d/kernels/velocityVerlet2.cl:1-26, dt = 1: the old-force
 * slot holds the previous acceleration. v <- (v + (a_old + f/m)/2) / (1 + xi/2); a = f/m - xi v;
 * x <- x + v + a/2; a_old <- a; f <- 0. */
static inline void NM(vv2_node)(long i, long np, real* points, real* vel, real* force, real* fold,
                                const real* masses, real xi) {
    V3 x = NM(load3)(points, np, i), v = NM(load3)(vel, np, i);
    const V3 f = NM(load3)(force, np, i), ao = NM(load3)(fold, np, i);
    const real m = masses[i];
    v = NM(vscale)(NM(vadd)(v, NM(vscale)(NM(vadd)(ao, NM(vdiv)(f, m)), (real)0.5)), (real)1.0 / (1 + xi / (real)2.0));
    const V3 a = NM(vsub)(NM(vdiv)(f, m), NM(vscale)(v, xi));
    x = NM(vadd)(NM(vadd)(x, v), NM(vscale)(a, (real)0.5));
    points[i] = x.x; points[np + i] = x.y; points[2 * np + i] = x.z;
    vel[i] = v.x; vel[np + i] = v.y; vel[2 * np + i] = v.z;
    fold[i] = a.x; fold[np + i] = a.y; fold[2 * np + i] = a.z;
    force[i] = 0; force[np + i] = 0; force[2 * np + i] = 0;
}

/* Sphere contact integrated over each tetra, nofluidx3d/kernels/InteractionSphereIntegral.cl:22-85:
 * a repulsive force density exp(-k (|x - c| - R)) (x - c)/|x - c| (c = (0, spos, 0)) evaluated at the
 * four-point Gauss rule of the tetra (the kernel's truncated coordinates 0.58541020 / 0.13819669)
 * and distributed to the corners with the linear shape functions, weighted by |det[p1-p4, p2-p4,
 * p3-p4]| / 4 as the kernel does. */
static inline V3 NM(si_density)(V3 x, real radius, real spos, real k) {
    const V3 r = NM(vsub)(x, NM(mk3)(0, spos, 0));
    const V3 n = NM(vdiv)(r, NM(vlen)(r));
    const real dis = NM(vlen)(r) - radius;
    return NM(vscale)(n, EXP(-k * dis));
}
static void NM(sphere_integral_tet)(long t, long np, long nt, const real* points, const unsigned* tets, real radius,
                                    real spos, real k, real* force) {
    const long ids[4] = {tets[t], tets[nt + t], tets[2 * nt + t], tets[3 * nt + t]};
    V3 p[4];
    for (int a = 0; a < 4; a++) p[a] = NM(load3)(points, np, ids[a]);
    const V3 r1 = NM(vsub)(p[0], p[3]), r2 = NM(vsub)(p[1], p[3]), r3 = NM(vsub)(p[2], p[3]);
    const real volume = FABS(NM(vdot)(r1, NM(vcross)(r2, r3)));
    const real al = (real)0.58541020, be = (real)0.13819669;
    const real xi[4][3] = {{al, be, be}, {be, al, be}, {be, be, al}, {be, be, be}};
    V3 fg[4];
    real N[4][4]; /* N[g][a]: shape function a at Gauss point g */
    for (int g = 0; g < 4; g++) {
        const real n4 = (real)1.0 - xi[g][0] - xi[g][1] - xi[g][2];
        const V3 x = NM(vadd)(NM(vadd)(NM(vadd)(NM(vscale)(p[0], xi[g][0]), NM(vscale)(p[1], xi[g][1])),
                                       NM(vscale)(p[2], xi[g][2])), NM(vscale)(p[3], n4));
        fg[g] = NM(si_density)(x, radius, spos, k);
        N[g][0] = xi[g][0]; N[g][1] = xi[g][1]; N[g][2] = xi[g][2]; N[g][3] = n4;
    }
    for (int a = 0; a < 4; a++) {
        V3 s = NM(vadd)(NM(vadd)(NM(vadd)(NM(vscale)(fg[0], N[0][a]), NM(vscale)(fg[1], N[1][a])),
                                 NM(vscale)(fg[2], N[2][a])), NM(vscale)(fg[3], N[3][a]));
        NM(add3)(force, np, ids[a], NM(vscale)(s, (real)0.25 * volume));
    }
}

/* Readout of the integrated sphere force, nofluidx3d/SimulationLegacy.py:260-273 (lattice units):
 * the force is recomputed into a zeroed buffer and -sum_i F_y(i) returned (node order, double). */
double NM(ora_sphere_integral_readout)(long np, long nt, const real* points, const unsigned* tets, real radius,
                                       real spos, real k) {
    real* buf = (real*)calloc((size_t)(3 * np), sizeof(real));
    for (long t = 0; t < nt; t++) NM(sphere_integral_tet)(t, np, nt, points, tets, radius, spos, k, buf);
    double s = 0;
    for (long i = 0; i < np; i++) s += (double)buf[np + i];
    free(buf);
    return -s;
}

/* Indenter-force readouts in lattice units (the host closures forceSI without the p0*L0^2 factor).
 * Plane, nofluidx3d/Simulation.py:146-153: sum_i k*max(y_i - wall, 0).
 * Sphere, nofluidx3d/Simulation.py:198-212: -sum_i [k*max(R - |x_i - c|, 0) * (x_i - c)/|x_i - c|]_y.
 * Accumulated in double in node order, like Python's sum over a float64 array. */
double NM(ora_plane_readout)(long np, const real* points, real wall, real k) {
    double s = 0;
    for (long i = 0; i < np; i++) {
        double dis = fmax((double)points[np + i] - (double)wall, 0.0);
        s += (double)k * dis;
    }
    return s;
}
double NM(ora_sphere_readout)(long np, const real* points, real radius, real spos, real k) {
    double s = 0;
    for (long i = 0; i < np; i++) {
        double rx = (double)points[i] - 0.0, ry = (double)points[np + i] - (double)spos;
        double rz = (double)points[2 * np + i] - 0.0;
        double len = sqrt(rx * rx + ry * ry + rz * rz);
        double dis = fmax((double)radius - len, 0.0);
        s += ((double)k * dis) * (ry / len);
    }
    return -s;
}

/* One time step in the order of nofluidx3d/Simulation.py:232-237 with the interactions registered as
 * element force, contacts (in the order given), velocity Verlet last (Simulation.py:227).
 * contact positions are evaluated by the caller for time t (the beforeTimeStep hook). */
void NM(ora_step)(const ora_problem* P, ora_state_p S, long t) {
    const long np = P->np, nt = P->nt;
    real* x = (real*)S->points;
    real* f = (real*)S->force;
    if (P->model == ORA_MODEL_VP)
        NM(ora_vp_force)(np, nt, x, P->tets, (const real*)P->edge, (const real*)S->vp_par, (real*)S->acc,
                         (real*)S->Fp, (real*)S->vonMises, (real*)S->pressure, f);
    else
        NM(ora_tet_force)(np, nt, x, P->tets, (const real*)P->edge, (const real*)P->vol, P->model,
                          (real)P->E, (real)P->nu, (real)P->mr, f);
    for (int c = 0; c < P->n_contacts; c++) {
        const ora_contact* C = &P->contacts[c];
        const real pos = (real)ora_contact_pos(C, (double)t);
        if (C->kind == ORA_SPHERE_INTEGRAL) {
            for (long e = 0; e < nt; e++)
                NM(sphere_integral_tet)(e, np, nt, x, P->tets, (real)C->radius, pos, (real)C->k, f);
            continue;
        }
        for (long i = 0; i < np; i++) {
            if (C->kind == ORA_SUBSTRATE) NM(substrate_node)(i, np, x, pos, (real)C->k, f);
            else if (C->kind == ORA_PLANE) NM(plane_node)(i, np, x, pos, (real)C->k, f);
            else NM(sphere_node)(i, np, x, (real)C->radius, pos, (real)C->k, f);
        }
    }
    if (P->integrator == 1) {
        for (long i = 0; i < np; i++)
            NM(vv2_node)(i, np, x, (real*)S->vel, f, (real*)S->fold, (const real*)P->masses, (real)P->xi);
        return;
    }
    for (long i = 0; i < np; i++)
        NM(vv_node)(i, np, x, (real*)S->vel, f, (real*)S->fold, (real)P->xi, P->fix_top_bottom);
}

double NM(ora_readout)(const ora_problem* P, ora_state_p S, long t) {
    if (P->record_contact < 0 || P->record_contact >= P->n_contacts) return 0.0;
    const ora_contact* C = &P->contacts[P->record_contact];
    const real pos = (real)ora_contact_pos(C, (double)t);
    if (C->kind == ORA_SPHERE) return NM(ora_sphere_readout)(P->np, (const real*)S->points, (real)C->radius, pos, (real)C->k);
    if (C->kind == ORA_PLANE) return NM(ora_plane_readout)(P->np, (const real*)S->points, pos, (real)C->k);
    if (C->kind == ORA_SPHERE_INTEGRAL)
        return NM(ora_sphere_integral_readout)(P->np, P->nt, (const real*)S->points, P->tets, (real)C->radius, pos,
                                               (real)C->k);
    return 0.0;
}

/* Serial run: nsteps steps from the state in S; at t = t0 and every record_every steps the curve
 * row (t, indentation, force) is written as in Simulation.run (Simulation.py:250-278). Returns
 * the number of rows written. */
long NM(ora_run)(const ora_problem* P, ora_state_p S, long t0, long nsteps, long record_every,
                 double* curve, long max_rows) {
    long rows = 0;
    if (record_every > 0 && curve && rows < max_rows) {
        ora_curve_row(P, t0, NM(ora_readout)(P, S, t0), curve + 3 * rows);
        rows++;
    }
    for (long s = 0; s < nsteps; s++) {
        const long t = t0 + s;
        NM(ora_step)(P, S, t);
        if (record_every > 0 && curve && ((t + 1 - t0) % record_every) == 0 && rows < max_rows) {
            ora_curve_row(P, t + 1, NM(ora_readout)(P, S, t + 1), curve + 3 * rows);
            rows++;
        }
    }
    return rows;
}

#undef V3
#undef M3
#undef NM
#undef NAME2
#undef NAME_
