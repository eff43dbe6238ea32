// Host emulation of the viscoplastic step's arithmetic — TEST INFRASTRUCTURE ONLY.
//
// The element law is the kernels' own header (nofluidx3d_gb300/csrc/nfx_math.cuh, whose
// functions compile for the host too), evaluated in FP32 on the displacement hi/lo parts exactly
// as the element pass forms them; the node update follows the node pass (FP32 velocity Verlet
// with the displacement carried by TwoSum, contacts in FP64). Corner forces are summed per node in
// double (the device sums them per tile in FP32 and adds the tile sums as 64-bit fixed point, an
// ulp-level difference). law64 = 1 evaluates the same law in double instead (the header with
// `real` for float, generated by the test into the build folder as nfx_math_f64.h); p64 = 1 keeps
// the plastic state P = Fp - I in double. Comparing the variants with the FP64 oracle separates the
// FP32 error of the law from that of the stored state. This exists to measure where FP32 loses
// accuracy; the reference has no such variants.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "nfx_math.cuh"
typedef double real;
#include "nfx_math_f64.h"

struct Contact {
    int kind;
    double k, radius, p0, v;
};

extern "C" int emu_run(long np, long nt, const double* P, const uint32_t* T, const double* vp, int ncont,
                       const Contact* cs, double xi, long nsteps, long every, int law64, int p64, double* out_pos,
                       double* curve) {
    // Dm^-1 and V0 as the planner builds them: double, stored as float
    std::vector<float> Dmi(9 * nt), V0(nt);
    for (long t = 0; t < nt; t++) {
        double M[9];
        const long n0 = T[t];
        for (int k = 0; k < 3; k++) {
            const long nk = T[(k + 1) * nt + t];
            for (int d = 0; d < 3; d++) M[3 * d + k] = P[d * np + nk] - P[d * np + n0];
        }
        const double A[9] = {M[4] * M[8] - M[5] * M[7], M[2] * M[7] - M[1] * M[8], M[1] * M[5] - M[2] * M[4],
                             M[5] * M[6] - M[3] * M[8], M[0] * M[8] - M[2] * M[6], M[2] * M[3] - M[0] * M[5],
                             M[3] * M[7] - M[4] * M[6], M[1] * M[6] - M[0] * M[7], M[0] * M[4] - M[1] * M[3]};
        const double det = M[0] * A[0] + M[1] * A[3] + M[2] * A[6];
        for (int k = 0; k < 9; k++) Dmi[9 * t + k] = (float)(A[k] / det);
        V0[t] = (float)(det / 6.0);
    }
    std::vector<float> Xh(3 * np), Xl(3 * np), uh(3 * np, 0.f), ul(3 * np, 0.f), v(3 * np, 0.f), fo(3 * np, 0.f);
    for (long i = 0; i < np; i++)
        for (int d = 0; d < 3; d++) {
            const double x = P[d * np + i];
            const float h = (float)x;
            Xh[3 * i + d] = h;
            Xl[3 * i + d] = (float)(x - (double)h);
        }
    std::vector<float> Pf(9 * nt, 0.f);
    std::vector<double> Pd(9 * nt, 0.0), cf(12 * nt);
    // node -> corner CSR, summed in a fixed order
    std::vector<long> off(np + 1, 0), adj(4 * nt);
    for (long i = 0; i < 4 * nt; i++) off[T[i] + 1]++;
    for (long i = 0; i < np; i++) off[i + 1] += off[i];
    {
        std::vector<long> f(off.begin(), off.end() - 1);
        for (long t = 0; t < nt; t++)
            for (int k = 0; k < 4; k++) adj[f[T[k * nt + t]]++] = 12 * t + 3 * k;
    }
    const nfx::VPParams pf{(float)vp[0], (float)vp[1], (float)vp[2], (float)vp[3],
                           (float)vp[4], (float)vp[5], (float)vp[6], (float)vp[7]};
    const nfxd::VPParams pd{vp[0], vp[1], vp[2], vp[3], vp[4], vp[5], vp[6], vp[7]};
    const float va = (float)((1 - 0.5 * xi) / (1 + 0.5 * xi)), hb = (float)(0.5 / (1 + 0.5 * xi)),
                dm = (float)(1 - 0.5 * xi);
    long row = 0;
    for (long s = 0; s <= nsteps; s++) {
        const bool last = s == nsteps;
        if (!last) {
#pragma omp parallel for schedule(static)
            for (long t = 0; t < nt; t++) {
                long n[4];
                for (int k = 0; k < 4; k++) n[k] = T[k * nt + t];
                if (law64) {
                    double d[3][3], Dd[9], Pp[9], dP[9], rate, f[4][3], vm, pr, jm1;
                    for (int k = 0; k < 3; k++)
                        for (int c = 0; c < 3; c++)
                            d[k][c] = ((double)uh[3 * n[k + 1] + c] - uh[3 * n[0] + c]) +
                                      ((double)ul[3 * n[k + 1] + c] - ul[3 * n[0] + c]);
                    for (int k = 0; k < 9; k++) Dd[k] = Dmi[9 * t + k];
                    for (int k = 0; k < 9; k++) Pp[k] = p64 ? Pd[9 * t + k] : (double)Pf[9 * t + k];
                    nfxd::vp_element(d[0], d[1], d[2], Dd, (double)V0[t], pd, Pp, 0.0, dP, rate, f, vm, pr, jm1);
                    for (int k = 0; k < 9; k++) {
                        if (p64) Pd[9 * t + k] += dP[k];
                        else Pf[9 * t + k] = (float)(Pf[9 * t + k] + dP[k]);
                    }
                    for (int k = 0; k < 4; k++)
                        for (int c = 0; c < 3; c++) cf[12 * t + 3 * k + c] = f[k][c];
                } else {
                    float d[3][3], Pp[9], dP[9], rate, f[4][3], vm, pr, jm1;
                    for (int k = 0; k < 3; k++)
                        for (int c = 0; c < 3; c++)
                            d[k][c] = (uh[3 * n[k + 1] + c] - uh[3 * n[0] + c]) + (ul[3 * n[k + 1] + c] - ul[3 * n[0] + c]);
                    for (int k = 0; k < 9; k++) Pp[k] = p64 ? (float)Pd[9 * t + k] : Pf[9 * t + k];
                    nfx::vp_element(d[0], d[1], d[2], &Dmi[9 * t], V0[t], pf, Pp, 0.f, dP, rate, f, vm, pr, jm1);
                    for (int k = 0; k < 9; k++) {
                        if (p64) Pd[9 * t + k] += (double)dP[k];
                        else Pf[9 * t + k] += dP[k];
                    }
                    for (int k = 0; k < 4; k++)
                        for (int c = 0; c < 3; c++) cf[12 * t + 3 * k + c] = f[k][c];
                }
            }
        }
        double ro = 0.0;
        const double tt = (double)s;
#pragma omp parallel for schedule(static) reduction(+ : ro)
        for (long i = 0; i < np; i++) {
            double acc[3] = {0, 0, 0};
            if (!last)
                for (long a = off[i]; a < off[i + 1]; a++)
                    for (int c = 0; c < 3; c++) acc[c] += cf[adj[a] + c];
            float f[3] = {(float)acc[0], (float)acc[1], (float)acc[2]};
            for (int ci = 0; ci < ncont; ci++) {
                const Contact& C = cs[ci];
                const double w = C.kind == 0 ? C.p0 : C.p0 - C.v * tt;
                double x[3];
                for (int c = 0; c < 3; c++) x[c] = (((double)Xh[3 * i + c] + Xl[3 * i + c]) + uh[3 * i + c]) + ul[3 * i + c];
                double fx = 0, fy = 0, fz = 0;
                if (C.kind == 0) {
                    fy = C.k * std::fmax(w - x[1], 0.0);
                } else if (C.kind == 1) {
                    fy = -C.k * std::fmax(x[1] - w, 0.0);
                } else {
                    const double rx = x[0], ry = x[1] - w, rz = x[2];
                    const double len = std::sqrt(rx * rx + ry * ry + rz * rz);
                    const double dis = std::fmax(C.radius - len, 0.0);
                    if (dis > 0) {
                        const double kd = C.k * dis;
                        fx = kd * (rx / len);
                        fy = kd * (ry / len);
                        fz = kd * (rz / len);
                    }
                }
                if (C.kind == 2) {
                    f[0] += (float)fx;
                    f[2] += (float)fz;
                }
                f[1] += (float)fy;
                if (ci == ncont - 1) ro += -fy;  // the indenter (last contact) readout
            }
            if (last) continue;
            for (int c = 0; c < 3; c++) {
                const float vv = va * v[3 * i + c] + hb * (f[c] + fo[3 * i + c]);
                nfx::df_add(uh[3 * i + c], ul[3 * i + c], dm * vv + 0.5f * f[c]);
                v[3 * i + c] = vv;
                fo[3 * i + c] = f[c];
            }
        }
        if (every > 0 && s % every == 0) {
            curve[3 * row] = (double)s;
            curve[3 * row + 1] = 0.0;
            curve[3 * row + 2] = ro;
            row++;
        }
    }
    for (long i = 0; i < np; i++)
        for (int c = 0; c < 3; c++)
            out_pos[3 * i + c] = (((double)Xh[3 * i + c] + Xl[3 * i + c]) + uh[3 * i + c]) + ul[3 * i + c];
    return (int)row;
}
