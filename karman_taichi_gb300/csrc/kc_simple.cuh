// Per-face and per-cell helpers of the SIMPLE assembly shared by the
// kernels of kc_simple.cu and the batched executor (kc_batch.cu): grid
// dimensions, the face-independent constants, the solid mask, which faces
// are unknowns, and the momentum rows of one u or v face.  Both units are
// compiled with -fmad=false, so a row computed by either is bit for bit the
// same (see kc_simple.cu for the reference behaviour and operation order).
#pragma once
#include "kc_common.cuh"

namespace kc {

struct Dims {
    int nx, ny;
    int NYu, NYv, NYp;
};
__host__ __device__ inline Dims dims_of(const kc_phys& P) { return {P.nx, P.ny, P.ny + 2, P.ny + 3, P.ny + 2}; }

// Subexpressions of the coefficient formulas that do not depend on the face,
// evaluated once on the host (the p' and wall constants with the same
// operation tree as the per-face expressions they replace, so those
// coefficients keep their bits; qdy, qdx and c0 serve the reduced momentum
// form).  On GB300
// FP64 arithmetic issues at a small fraction of the FP32 rate: a division
// per face that need not be there costs more than the face's memory traffic.
struct SimpleK {
    double mdy_dx;   // mu * dy / dx
    double mdx_dy;   // mu * dx / dy
    double qdy;      // 0.5 * rho * 0.5 * dy
    double qdx;      // 0.5 * rho * 0.5 * dx
    double c0;       // 2 mu dy / dx + 2 mu dx / dy + rho dx dy / dt (the velocity-free part of aP)
    double rdt;      // rho * dx * dy / dt
    double wall_x;   // 2 * mu * dx / dy
    double wall_y;   // 2 * mu * dy / dx
    double nrdy2;    // -rho * dy * dy
    double nrdx2;    // -rho * dx * dx
    double one_m_am; // 1 - alpha_m
};
inline SimpleK consts_of(const kc_phys& P) {
    SimpleK K;
    K.mdy_dx = P.mu * P.dy / P.dx;
    K.mdx_dy = P.mu * P.dx / P.dy;
    K.qdy = 0.5 * P.rho * 0.5 * P.dy;
    K.qdx = 0.5 * P.rho * 0.5 * P.dx;
    K.rdt = P.rho * P.dx * P.dy / P.dt;
    K.c0 = (2 * K.mdy_dx + 2 * K.mdx_dy) + K.rdt;
    K.wall_x = 2 * P.mu * P.dx / P.dy;
    K.wall_y = 2 * P.mu * P.dy / P.dx;
    K.nrdy2 = -P.rho * P.dy * P.dy;
    K.nrdx2 = -P.rho * P.dx * P.dx;
    K.one_m_am = 1 - P.alpha_m;
    return K;
}

struct Solid {
    const unsigned char* s;
    int NYp;
    __device__ __forceinline__ bool cell(int i, int j) const { return s && s[(long long)i * NYp + j]; }
    // u face (i,j) lies between cells (i-1,j) and (i,j)
    __device__ __forceinline__ bool bu(int i, int j) const { return cell(i - 1, j) || cell(i, j); }
    // v face (i,j) lies between cells (i,j-1) and (i,j)
    __device__ __forceinline__ bool bv(int i, int j) const { return cell(i, j - 1) || cell(i, j); }
};

__device__ __forceinline__ bool unk_u(const kc_phys& P, const Solid& S, int i, int j) {
    if (i < 2 || i > P.nx || j < 1 || j > P.ny) return false;
    return P.mode != KC_MODE_CHANNEL || !S.bu(i, j);
}
__device__ __forceinline__ bool unk_v(const kc_phys& P, const Solid& S, int i, int j) {
    if (i < 1 || i > P.nx || j < 2 || j > P.ny) return false;
    return P.mode != KC_MODE_CHANNEL || !S.bv(i, j);
}

// ---- momentum ---------------------------------------------------------------
__device__ __forceinline__ void u_row(const kc_phys& P, const SimpleK& K, const Dims& D, const Solid& S,
                                      const double* u, const double* v, const double* p, const double* u0, int i,
                                      int j, double (&c)[5], double& b) {
    c[0] = c[1] = c[2] = c[3] = c[4] = 0.0;
    b = 0.0;
    const int nx = D.nx, ny = D.ny;
    if (i < 2 || i > nx || j < 1 || j > ny) return;
    if (P.mode == KC_MODE_CHANNEL && S.bu(i, j)) {
        c[0] = 1.0;
        return;
    }
    const double mu = P.mu, dx = P.dx, dy = P.dy;
#define U_(a, bb) u[(long long)(a) * D.NYu + (bb)]
#define V_(a, bb) v[(long long)(a) * D.NYv + (bb)]
#define P_(a, bb) p[(long long)(a) * D.NYp + (bb)]
    const double ui = U_(i, j), uw = U_(i - 1, j), ue = U_(i + 1, j);
    const double vnw = V_(i - 1, j + 1), vne = V_(i, j + 1), vsw = V_(i - 1, j), vse = V_(i, j);
    const double sw = ui + uw, se = ui + ue, sn = vnw + vne, ss = vsw + vse;
    // aW = -(mu dy/dx + rho/4 sw dy), aE = -(mu dy/dx - rho/4 se dy), aN / aS alike in x;
    // aP = -(aW + aE + aN + aS) + rho/2 (se - sw) dy + rho/2 (sn - ss) dx + rho dx dy / dt, which
    // reduces exactly to c0 + rho/4 (se - sw) dy + rho/4 (sn - ss) dx
    double aW = -fma(K.qdy, sw, K.mdy_dx);
    double aE = fma(K.qdy, se, -K.mdy_dx);
    double aN = fma(K.qdx, sn, -K.mdx_dy);
    double aS = -fma(K.qdx, ss, K.mdx_dy);
    double aP = fma(K.qdx, sn - ss, fma(K.qdy, se - sw, K.c0));
    double bb = fma(P_(i - 1, j) - P_(i, j), dy, K.rdt * u0[(long long)i * D.NYu + j]);
    if (P.mode == KC_MODE_CHANNEL) {
        const double wall = K.wall_x;
        if (i == 2) {
            bb += -aW * P.U;
            aW = 0.0;
        } else if (S.bu(i - 1, j)) {
            aW = 0.0;
        }
        if (i == nx) {
            aP = aP + aE;
            aE = 0.0;
        } else if (S.bu(i + 1, j)) {
            aE = 0.0;
        }
        if (j == 1 || S.bu(i, j - 1)) {
            aP = aP + (aS + wall);
            aS = 0.0;
        }
        if (j == ny || S.bu(i, j + 1)) {
            aP = aP + (aN + wall);
            aN = 0.0;
        }
    } else {
        // set_bc, simple.py:177-207 (w, e, then south/north sliding walls)
        if (i == 2) {
            bb += -aW * P.bc[0][0];
            aW = 0.0;
        }
        if (i == nx) {
            bb += -aE * P.bc[1][0];
            aE = 0.0;
        }
        if (j == 1) {
            bb += 2 * mu * P.bc[3][1] * dx / dy;
            aP += (aS + K.wall_x);
            aS = 0.0;
        }
        if (j == ny) {
            bb += 2 * mu * P.bc[2][1] * dx / dy;
            aP += (aN + K.wall_x);
            aN = 0.0;
        }
    }
    c[0] = aP;
    c[1] = aW;
    c[2] = aE;
    c[3] = aN;
    c[4] = aS;
    b = bb;
}

__device__ __forceinline__ void v_row(const kc_phys& P, const SimpleK& K, const Dims& D, const Solid& S,
                                      const double* u, const double* v, const double* p, const double* v0, int i,
                                      int j, double (&c)[5], double& b) {
    c[0] = c[1] = c[2] = c[3] = c[4] = 0.0;
    b = 0.0;
    const int nx = D.nx, ny = D.ny;
    if (i < 1 || i > nx || j < 2 || j > ny) return;
    if (P.mode == KC_MODE_CHANNEL && S.bv(i, j)) {
        c[0] = 1.0;
        return;
    }
    const double mu = P.mu, dx = P.dx, dy = P.dy;
    const double uc = U_(i, j), us = U_(i, j - 1), uec = U_(i + 1, j), ues = U_(i + 1, j - 1);
    const double vc = V_(i, j), vn = V_(i, j + 1), vs = V_(i, j - 1);
    const double sw = uc + us, se = ues + uec, sn = vn + vc, ss = vs + vc;
    // the reduced form of u_row
    double aW = -fma(K.qdy, sw, K.mdy_dx);
    double aE = fma(K.qdy, se, -K.mdy_dx);
    double aN = fma(K.qdx, sn, -K.mdx_dy);
    double aS = -fma(K.qdx, ss, K.mdx_dy);
    double aP = fma(K.qdx, sn - ss, fma(K.qdy, se - sw, K.c0));
    double bb = fma(P_(i, j - 1) - P_(i, j), dx, K.rdt * v0[(long long)i * D.NYv + j]);
    if (P.mode == KC_MODE_CHANNEL) {
        const double wall = K.wall_y;
        if (j == 2 || S.bv(i, j - 1)) aS = 0.0;
        if (j == ny || S.bv(i, j + 1)) aN = 0.0;
        if (i == 1 || S.bv(i - 1, j)) {
            aP = aP + (aW + wall);
            aW = 0.0;
        }
        if (i == nx) {
            aP = aP + aE;
            aE = 0.0;
        } else if (S.bv(i + 1, j)) {
            aP = aP + (aE + wall);
            aE = 0.0;
        }
    } else {
        // set_bc, simple.py:188-216 (s, n, then west/east sliding walls)
        if (j == 2) {
            bb += -aS * P.bc[3][0];
            aS = 0.0;
        }
        if (j == ny) {
            bb += -aN * P.bc[2][0];
            aN = 0.0;
        }
        if (i == 1) {
            bb += 2 * mu * P.bc[0][1] * dy / dx;
            aP += (aW + K.wall_y);
            aW = 0.0;
        }
        if (i == nx) {
            bb += 2 * mu * P.bc[1][1] * dy / dx;
            aP += ((P.mode == KC_MODE_BICGSIMP ? aE : aW) + K.wall_y);
            aE = 0.0;
        }
    }
    c[0] = aP;
    c[1] = aW;
    c[2] = aE;
    c[3] = aN;
    c[4] = aS;
    b = bb;
}
#undef U_
#undef V_
#undef P_

}  // namespace kc
