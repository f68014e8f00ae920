// Finite-volume kernels of the SIMPLE hot path (FP64).
//
// Assembly is race-free without atomics: a face pass computes each interior
// face's coupling coefficient and explicit flux once (from the side of its
// first cell; the second cell gets the negated flux), a boundary pass does the
// same per boundary record, and a cell pass gathers over the cell's faces in
// the reference's Cell[i].face[] order, writing its own matrix row, diagonal
// and right-hand side.  Expression order inside each formula follows the
// reference source line it cites, so the two codes differ by rounding only
// where a sum is split between the face and the cell pass.
#include "fv.hpp"

#include <cmath>

namespace sysu {

namespace {

constexpr int NB = FV_BLOCK;
constexpr double SMALL = 1.e-16;  // BasicType.h:15

inline int nblk(int n) { return (n + NB - 1) / NB; }
inline int nblk_capped(int n, int cap) {
    int b = nblk(n);
    return b < 1 ? 1 : (b > cap ? cap : b);
}

__device__ __forceinline__ double cmin(double x, double y) { return x < y ? x : y; }  // CYCASMIN
__device__ __forceinline__ double cmax(double x, double y) { return x > y ? x : y; }  // CYCASMAX

__device__ __forceinline__ long sell_pos(const SellView &A, int row, int k) {
    return (long)A.sl_ptr[row >> 5] + (long)k * 32 + (row & 31);
}

// Last-block reduction into rs.out[slot[k]] (assignment).
template <int NV>
__device__ __forceinline__ void reduce_to_slots(double (&v)[NV], const int (&slot)[NV], RedScratch rs) {
    __shared__ double smem[NV * (NB / 32)];
    __shared__ int s_last;
    block_sum<NV>(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) rs.partials[(size_t)slot[k] * rs.max_blocks + blockIdx.x] = v[k];
        __threadfence();
        unsigned int t = atomicAdd(rs.ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        if (threadIdx.x < 32) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                double s = warp_sum_partials(rs.partials + (size_t)slot[k] * rs.max_blocks, gridDim.x);
                if (threadIdx.x == 0) rs.out[slot[k]] = s;
            }
        }
        if (threadIdx.x == 0) *rs.ticket = 0u;
    }
}

// ---------------------------------------------------------------------------
// SetBCVelocity, navier_bc.cpp:8-108
__global__ void k_bc_velocity(DomView d, const double *R, const double *U, const double *V, const double *W,
                              double *BRo, double *BU, double *BV, double *BW, int has_outlet, RedScratch rs) {
    double v[3] = {0.0, 0.0, 0.0};
    for (int b = blockIdx.x * NB + threadIdx.x; b < d.B; b += gridDim.x * NB) {
        int ic = d.bcell[b];
        int f = d.F + b;
        int ty = d.btype1[b];
        double br, bu, bv, bw;
        if (ty == 1) {
            br = R[ic]; bu = 0.; bv = 0.; bw = 0.;
        } else if (ty == 2) {
            br = d.bin[4 * d.B + b];
            bu = d.bin[0 * d.B + b];
            bv = d.bin[1 * d.B + b];
            bw = d.bin[2 * d.B + b];
        } else if (ty == 3) {
            br = R[ic]; bu = U[ic]; bv = V[ic]; bw = W[ic];
        } else {  // 4: symmetry
            double a = d.farea[f];
            double s1 = d.fn[f] / a, s2 = d.fn[d.nf + f] / a, s3 = d.fn[2 * d.nf + f] / a;
            double un = U[ic] * s1 + V[ic] * s2 + W[ic] * s3;
            bu = U[ic] - un * s1;
            bv = V[ic] - un * s2;
            bw = W[ic] - un * s3;
            br = R[ic];
        }
        BRo[b] = br; BU[b] = bu; BV[b] = bv; BW[b] = bw;
        if (has_outlet) {
            double m = br * (bu * d.fn[f] + bv * d.fn[d.nf + f] + bw * d.fn[2 * d.nf + f]);
            if (ty == 2) v[0] += m;
            else if (ty == 3) { v[1] += m; v[2] += br * d.bquirk_area[b]; }
        }
    }
    if (has_outlet) {
        const int slots[3] = {RED_MASS_IN, RED_MASS_OUT, RED_AREA_OUT};
        reduce_to_slots<3>(v, slots, rs);
    }
}

// outlet rescaling, navier_bc.cpp:87-107
__global__ void k_bc_outlet(DomView d, double *BU, double *BV, double *BW, const double *red_out) {
    int b = blockIdx.x * NB + threadIdx.x;
    if (b >= d.B || d.btype1[b] != 3) return;
    double min_ = red_out[RED_MASS_IN], mout = red_out[RED_MASS_OUT], aout = red_out[RED_AREA_OUT];
    if (fabs(mout) > SMALL) {
        double rate = -min_ / mout;
        BU[b] *= rate; BV[b] *= rate; BW[b] *= rate;
    } else {
        double rate = (-min_ - mout) / aout;
        int f = d.F + b;
        double a = d.farea[f];
        BU[b] += rate * d.fn[f] / a;
        BV[b] += rate * d.fn[d.nf + f] / a;
        BW[b] += rate * d.fn[2 * d.nf + f] / a;
    }
}

// Bphi[b] = phi(cell of b): SetBCPressure / SetBCDeltaP (navier_bc.cpp:110-162)
__global__ void k_bnd_from_cell(DomView d, const double *phi, double *Bphi) {
    int b = blockIdx.x * NB + threadIdx.x;
    if (b < d.B) Bphi[b] = phi[d.bcell[b]];
}

// ---------------------------------------------------------------------------
// Green-Gauss gradient, BasicSolver.cpp:29-63, as a per-cell gather.
struct GradPtrs {
    const double *phi[4];
    const double *Bphi[4];
    double *grad[4];
};

// Green-Gauss gradient of NF fields, one thread per cell over its slots in
// SELL-32 order: the slot words (face id, neighbour) of all six slots are loaded
// first, so each cell waits for two rounds of loads instead of three per face.
// The arithmetic and the summation order are those of the per-face form
// (phi_f = lambda phi_c1 + (1 - lambda) phi_c2, negated for the face's cell2).
template <int NF>
__global__ void __launch_bounds__(NB) k_gradient_v(DomView d, GradPtrs p) {
    const double *phi[NF];
    const double *Bphi[NF];
    double *grad[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) { phi[k] = p.phi[k]; Bphi[k] = p.Bphi[k]; grad[k] = p.grad[k]; }
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    const int sl = i >> 5, lane = i & 31;
    const int base = d.ss_ptr[sl] + lane, w = d.ss_w[sl];
    int fs[6], ns[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        fs[j] = -1;
        ns[j] = 0;
        if (j < w) {
            fs[j] = __ldg(d.ss_f + base + 32 * j);
            ns[j] = __ldg(d.ss_n + base + 32 * j);
        }
    }
    double own[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) own[k] = __ldg(phi[k] + i);
    double g[NF][3];
#pragma unroll
    for (int k = 0; k < NF; ++k) g[k][0] = g[k][1] = g[k][2] = 0.;
    const int nf = d.nf;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const int f = fs[j];
        if (f < 0) continue;
        const int nb = ns[j];
        double n0 = __ldg(d.fn + f), n1 = __ldg(d.fn + nf + f), n2 = __ldg(d.fn + 2 * nf + f);
        double pf[NF];
        if (nb >= 0 && (nb & SS_BND)) {
            const int b = nb & ~SS_BND;
#pragma unroll
            for (int k = 0; k < NF; ++k) pf[k] = __ldg(Bphi[k] + b);
        } else {
            const bool c2side = nb < 0;
            const int o = nb & 0x7FFFFFFF;
            double lam = __ldg(d.flam + f);
            double lam2 = 1. - lam;
#pragma unroll
            for (int k = 0; k < NF; ++k) {
                double po = __ldg(phi[k] + o);
                pf[k] = c2side ? -(lam * po + lam2 * own[k]) : lam * own[k] + lam2 * po;
            }
        }
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            g[k][0] += pf[k] * n0;
            g[k][1] += pf[k] * n1;
            g[k][2] += pf[k] * n2;
        }
    }
    // one FP64 division per cell instead of 3 NF (the FP64 pipe bounds this
    // kernel on GB300); the reference divides each component (BasicSolver.cpp:72),
    // the results differ by at most an ulp
    const double rvol = 1.0 / d.vol[i];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        grad[k][i] = g[k][0] * rvol;
        grad[k][d.nc + i] = g[k][1] * rvol;
        grad[k][2 * d.nc + i] = g[k][2] * rvol;
    }
}

// ---------------------------------------------------------------------------
// Least-squares gradients (an option beside the reference's Green-Gauss one):
// grad phi_c = M^-1 sum_j w_j d_j (phi_j - phi_c) over the cell's faces, phi_j the
// neighbour's value or the boundary value, d_j from the cell centroid to the
// neighbour's centroid or the boundary face's, w_j = 1 / |d_j|^2.  Exact for
// linear fields.  The geometry part c_j = M^-1 w_j d_j is computed once.
__device__ __forceinline__ void lsq_offset(const DomView &d, int i, int f, int nb, double &d0, double &d1,
                                           double &d2) {
    double x0, x1, x2;
    if (nb >= 0 && (nb & SS_BND)) {
        x0 = d.fx[f];
        x1 = d.fx[d.nf + f];
        x2 = d.fx[2 * d.nf + f];
    } else {
        const int o = nb & 0x7FFFFFFF;
        x0 = d.cx[o];
        x1 = d.cx[d.nc + o];
        x2 = d.cx[2 * d.nc + o];
    }
    d0 = x0 - d.cx[i];
    d1 = x1 - d.cx[d.nc + i];
    d2 = x2 - d.cx[2 * d.nc + i];
}

__global__ void __launch_bounds__(NB) k_lsq_setup(DomView d, double *c) {
    const int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    const int base = d.ss_ptr[i >> 5] + (i & 31), w = d.ss_w[i >> 5];
    double a = 0, b = 0, cc = 0, dd = 0, e = 0, ff = 0;  // M = [a b cc; b dd e; cc e ff]
    for (int j = 0; j < w; ++j) {
        const int f = d.ss_f[base + 32 * j];
        if (f < 0) continue;
        double d0, d1, d2;
        lsq_offset(d, i, f, d.ss_n[base + 32 * j], d0, d1, d2);
        const double wt = 1.0 / (d0 * d0 + d1 * d1 + d2 * d2);
        a += wt * d0 * d0;
        b += wt * d0 * d1;
        cc += wt * d0 * d2;
        dd += wt * d1 * d1;
        e += wt * d1 * d2;
        ff += wt * d2 * d2;
    }
    // symmetric inverse by cofactors
    const double A00 = dd * ff - e * e, A01 = cc * e - b * ff, A02 = b * e - cc * dd;
    const double A11 = a * ff - cc * cc, A12 = b * cc - a * e, A22 = a * dd - b * b;
    const double det = a * A00 + b * A01 + cc * A02;
    const double tr = a + dd + ff;
    const bool ok = isfinite(det) && fabs(det) > 1e-12 * tr * tr * tr;
    const double r = ok ? 1.0 / det : 0.0;
    for (int j = 0; j < w; ++j) {
        const int pos = base + 32 * j;
        const int f = d.ss_f[pos];
        double c0 = 0, c1 = 0, c2 = 0;
        if (f >= 0 && ok) {
            double d0, d1, d2;
            lsq_offset(d, i, f, d.ss_n[pos], d0, d1, d2);
            const double wt = 1.0 / (d0 * d0 + d1 * d1 + d2 * d2);
            c0 = r * wt * (A00 * d0 + A01 * d1 + A02 * d2);
            c1 = r * wt * (A01 * d0 + A11 * d1 + A12 * d2);
            c2 = r * wt * (A02 * d0 + A12 * d1 + A22 * d2);
        }
        c[pos] = c0;
        c[d.ss_tot + pos] = c1;
        c[2 * d.ss_tot + pos] = c2;
    }
}

template <int NF>
__global__ void __launch_bounds__(NB) k_gradient_lsq(DomView d, GradPtrs p) {
    const int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    const int base = d.ss_ptr[i >> 5] + (i & 31), w = d.ss_w[i >> 5];
    double own[NF], g[NF][3];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        own[k] = __ldg(p.phi[k] + i);
        g[k][0] = g[k][1] = g[k][2] = 0.;
    }
    for (int j = 0; j < w; ++j) {
        const int pos = base + 32 * j;
        const int f = __ldg(d.ss_f + pos);
        if (f < 0) continue;
        const int nb = __ldg(d.ss_n + pos);
        const double c0 = __ldg(d.lsq_c + pos), c1 = __ldg(d.lsq_c + d.ss_tot + pos),
                     c2 = __ldg(d.lsq_c + 2 * d.ss_tot + pos);
        const bool bnd = nb >= 0 && (nb & SS_BND);
        const int o = bnd ? (nb & ~SS_BND) : (nb & 0x7FFFFFFF);
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            const double dphi = (bnd ? __ldg(p.Bphi[k] + o) : __ldg(p.phi[k] + o)) - own[k];
            g[k][0] = fma(c0, dphi, g[k][0]);
            g[k][1] = fma(c1, dphi, g[k][1]);
            g[k][2] = fma(c2, dphi, g[k][2]);
        }
    }
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        p.grad[k][i] = g[k][0];
        p.grad[k][d.nc + i] = g[k][1];
        p.grad[k][2 * d.nc + i] = g[k][2];
    }
}

// ---------------------------------------------------------------------------
// Limiters, BasicSolver.cpp:88-288
__device__ __forceinline__ double barth_fun(double us, double umin, double umax) {
    if (us > 1.0e-10) return cmin(1., umax / us);
    if (us < -1.0e-10) return cmin(1., umin / us);
    return 1.;
}

// WENO: inverse-|grad|^2 weighted average of own and neighbour gradients
__global__ void k_limiter_weno(DomView d, const double *grad, double *out) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    int n = d.nc;
    double ss = 0., t0 = 0., t1 = 0., t2 = 0.;
    for (int s = d.cs_ptr[i]; s < d.cs_ptr[i + 1]; ++s) {
        int f = d.cs_face[s];
        if (f >= d.F) continue;
        int ic = d.fc1[f] == i ? d.fc2[f] : d.fc1[f];
        double g0 = grad[ic], g1 = grad[n + ic], g2 = grad[2 * n + ic];
        double wei = 1. / (g0 * g0 + g1 * g1 + g2 * g2 + 1.e-16);
        ss += wei;
        t0 += wei * g0;
        t1 += wei * g1;
        t2 += wei * g2;
    }
    double g0 = grad[i], g1 = grad[n + i], g2 = grad[2 * n + i];
    double wei = 1. / (g0 * g0 + g1 * g1 + g2 * g2 + 1.e-16);
    ss += wei;
    t0 += wei * g0;
    t1 += wei * g1;
    t2 += wei * g2;
    out[i] = t0 / ss;
    out[n + i] = t1 / ss;
    out[2 * n + i] = t2 / ss;
}

__global__ void k_copy3(int n, const double *src, double *dst) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i < 3 * n) dst[i] = src[i];
}

// Barth: neighbour-cell bounds, vertex extrapolation
__global__ void k_limiter_barth(DomView d, const double *phi, double *grad) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    int n = d.nc;
    double umax = phi[i], umin = phi[i];
    for (int s = d.cs_ptr[i]; s < d.cs_ptr[i + 1]; ++s) {
        int f = d.cs_face[s];
        if (f >= d.F) continue;
        int ic = d.fc1[f] == i ? d.fc2[f] : d.fc1[f];
        umax = cmax(umax, phi[ic]);
        umin = cmin(umin, phi[ic]);
    }
    umax -= phi[i];
    umin -= phi[i];
    double g0 = grad[i], g1 = grad[n + i], g2 = grad[2 * n + i];
    double fi = 10.;
    for (int j = 0; j < 8; ++j) {
        int iv = d.cvert[j * n + i];
        double dx = d.vx[3 * iv] - d.cx[i];
        double dy = d.vx[3 * iv + 1] - d.cx[n + i];
        double dz = d.vx[3 * iv + 2] - d.cx[2 * n + i];
        double us = g0 * dx + g1 * dy + g2 * dz;
        fi = cmin(fi, barth_fun(us, umin, umax));
    }
    grad[i] = fi * g0;
    grad[n + i] = fi * g1;
    grad[2 * n + i] = fi * g2;
}

// MLP: vertex bounds over the cells around each vertex
__global__ void k_vertex_minmax(DomView d, const double *phi, double *vmax, double *vmin) {
    int v = blockIdx.x * NB + threadIdx.x;
    if (v >= d.nv) return;
    double mx = -1.e8, mn = 1.e8;
    for (int k = d.vc_ptr[v]; k < d.vc_ptr[v + 1]; ++k) {
        double p = phi[d.vc_cell[k]];
        mx = cmax(mx, p);
        mn = cmin(mn, p);
    }
    vmax[v] = mx;
    vmin[v] = mn;
}

__global__ void k_limiter_mlp(DomView d, const double *phi, const double *vmax, const double *vmin, double *grad) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    int n = d.nc;
    double g0 = grad[i], g1 = grad[n + i], g2 = grad[2 * n + i];
    double fi = 10.;
    for (int j = 0; j < 8; ++j) {
        int iv = d.cvert[j * n + i];
        double umax = vmax[iv] - phi[i];
        double umin = vmin[iv] - phi[i];
        double dx = d.vx[3 * iv] - d.cx[i];
        double dy = d.vx[3 * iv + 1] - d.cx[n + i];
        double dz = d.vx[3 * iv + 2] - d.cx[2 * n + i];
        double us = g0 * dx + g1 * dy + g2 * dz;
        fi = cmin(fi, barth_fun(us, umin, umax));
    }
    grad[i] = fi * g0;
    grad[n + i] = fi * g1;
    grad[2 * n + i] = fi * g2;
}

// ---------------------------------------------------------------------------
// Momentum, navier_velocity.cpp:77-357.  Interior face pass, from cell1's side.
template <bool HYB>  // the hybrid scheme: a compile-time branch, so the default kernel does no extra work
__global__ void k_mom_face(DomView d, MomArgs a) {
    int f = blockIdx.x * NB + threadIdx.x;
    if (f >= d.F) return;
    const int nc = d.nc, nf = d.nf;
    int c1 = d.fc1[f], c2 = d.fc2[f];
    double lambda = d.flam[f];
    double lambda2 = 1. - lambda;
    double sav1 = d.fn[f], sav2 = d.fn[nf + f], sav3 = d.fn[2 * nf + f];
    double RU = a.RUFace[f];
    double Visc = lambda * (a.VisLam[c1] + a.VisTur[c1]) + lambda2 * (a.VisLam[c2] + a.VisTur[c2]);
    double dudx = lambda * a.dU[c1] + lambda2 * a.dU[c2];
    double dudy = lambda * a.dU[nc + c1] + lambda2 * a.dU[nc + c2];
    double dudz = lambda * a.dU[2 * nc + c1] + lambda2 * a.dU[2 * nc + c2];
    double dvdx = lambda * a.dV[c1] + lambda2 * a.dV[c2];
    double dvdy = lambda * a.dV[nc + c1] + lambda2 * a.dV[nc + c2];
    double dvdz = lambda * a.dV[2 * nc + c1] + lambda2 * a.dV[2 * nc + c2];
    double dwdx = lambda * a.dW[c1] + lambda2 * a.dW[c2];
    double dwdy = lambda * a.dW[nc + c1] + lambda2 * a.dW[nc + c2];
    double dwdz = lambda * a.dW[2 * nc + c1] + lambda2 * a.dW[2 * nc + c2];
    double D = Visc * d.frl[f];
    // deferred correction to linear upwind (:269-295); none with the hybrid scheme
    double fcs0 = 0., fcs1 = 0., fcs2 = 0.;
    if (!HYB) {
        int up = RU > 0. ? c1 : c2;
        double dx0 = d.fx[f] - d.cx[up], dx1 = d.fx[nf + f] - d.cx[nc + up], dx2 = d.fx[2 * nf + f] - d.cx[2 * nc + up];
        double ufi = a.U[up], vfi = a.V[up], wfi = a.W[up];
        double ufh = ufi + (a.dU[up] * dx0 + a.dU[nc + up] * dx1 + a.dU[2 * nc + up] * dx2);
        double vfh = vfi + (a.dV[up] * dx0 + a.dV[nc + up] * dx1 + a.dV[2 * nc + up] * dx2);
        double wfh = wfi + (a.dW[up] * dx0 + a.dW[nc + up] * dx1 + a.dW[2 * nc + up] * dx2);
        fcs0 = RU * (ufh - ufi);
        fcs1 = RU * (vfh - vfi);
        fcs2 = RU * (wfh - wfi);
    }
    // explicit part of the stress (:302-309) and non-orthogonal correction (:313-316)
    double fde0 = ((dudx + dudx) * sav1 + (dudy + dvdx) * sav2 + (dudz + dwdx) * sav3) * Visc;
    double fde1 = ((dvdx + dudy) * sav1 + (dvdy + dvdy) * sav2 + (dvdz + dwdy) * sav3) * Visc;
    double fde2 = ((dwdx + dudz) * sav1 + (dwdy + dvdz) * sav2 + (dwdz + dwdz) * sav3) * Visc;
    double dxc0 = d.cx[c2] - d.cx[c1], dxc1 = d.cx[nc + c2] - d.cx[nc + c1], dxc2 = d.cx[2 * nc + c2] - d.cx[2 * nc + c1];
    double fdi0 = D * (dudx * dxc0 + dudy * dxc1 + dudz * dxc2);
    double fdi1 = D * (dvdx * dxc0 + dvdy * dxc1 + dvdz * dxc2);
    double fdi2 = D * (dwdx * dxc0 + dwdy * dxc1 + dwdz * dxc2);
    a.fD[f] = D;
    a.fE[f] = fde0 - fdi0 - fcs0;
    a.fE[d.F + f] = fde1 - fdi1 - fcs1;
    a.fE[2 * d.F + f] = fde2 - fdi2 - fcs2;
}

// boundary pass (:126-223)
__global__ void k_mom_bnd(DomView d, MomArgs a) {
    int b = blockIdx.x * NB + threadIdx.x;
    if (b >= d.B) return;
    const int nc = d.nc, nf = d.nf;
    int i = d.bcell[b];
    int f = d.F + b;
    int ty = d.btype1[b];
    double sav1 = d.fn[f], sav2 = d.fn[nf + f], sav3 = d.fn[2 * nf + f];
    double RU = a.RUFace[f];
    double Visc = a.VisLam[i] + a.VisTur[i];
    double dudx = a.dU[i], dudy = a.dU[nc + i], dudz = a.dU[2 * nc + i];
    double dvdx = a.dV[i], dvdy = a.dV[nc + i], dvdz = a.dV[2 * nc + i];
    double dwdx = a.dW[i], dwdy = a.dW[nc + i], dwdz = a.dW[2 * nc + i];
    double dxc0 = d.fx[f] - d.cx[i], dxc1 = d.fx[nf + f] - d.cx[nc + i], dxc2 = d.fx[2 * nf + f] - d.cx[2 * nc + i];
    double app = 0., fde0, fde1, fde2, fdi0, fdi1, fdi2, fcs0 = 0., fcs1 = 0., fcs2 = 0.;
    double VAL = Visc * d.frl[f];
    app += VAL;
    if (ty == 1) {
        double u = a.U[i], v = a.V[i], w = a.W[i];
        fde0 = VAL * u; fde1 = VAL * v; fde2 = VAL * w;
        fdi0 = VAL * u; fdi1 = VAL * v; fdi2 = VAL * w;
    } else {
        fde0 = ((dudx + dudx) * sav1 + (dudy + dvdx) * sav2 + (dudz + dwdx) * sav3) * Visc;
        fde1 = ((dvdx + dudy) * sav1 + (dvdy + dvdy) * sav2 + (dvdz + dwdy) * sav3) * Visc;
        fde2 = ((dwdx + dudz) * sav1 + (dwdy + dvdz) * sav2 + (dwdz + dwdz) * sav3) * Visc;
        fdi0 = VAL * (dudx * dxc0 + dudy * dxc1 + dudz * dxc2 - a.BU[b]);
        fdi1 = VAL * (dvdx * dxc0 + dvdy * dxc1 + dvdz * dxc2 - a.BV[b]);
        fdi2 = VAL * (dwdx * dxc0 + dwdy * dxc1 + dwdz * dxc2 - a.BW[b]);
    }
    if (ty == 2 || ty == 3) {
        double fl = cmin(RU, 0.0);
        app -= fl;
        fcs0 = fl * a.BU[b];
        fcs1 = fl * a.BV[b];
        fcs2 = fl * a.BW[b];
    }
    if (ty < 1 || ty > 4) atomicOr(a.flags, 1);
    a.bapp[b] = app;
    a.bsrc[b] = fde0 - fdi0 - fcs0;
    a.bsrc[d.B + b] = fde1 - fdi1 - fcs1;
    a.bsrc[2 * d.B + b] = fde2 - fdi2 - fcs2;
}

// cell pass (:95-355): diagonal, off-diagonals, Apr and the three RHS
template <bool HYB>
__global__ void k_mom_cell(DomView d, MomArgs a) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    const int nc = d.nc;
    double app = 0., su = 0., sv = 0., sw = 0.;
    if (a.tscheme) {  // unsteady terms first, navier_velocity.cpp:103-118
        double coef = a.R[i] / a.dt * d.vol[i];
        if (a.tscheme == 1) {
            app += coef;
            su += coef * a.Unp[i];
            sv += coef * a.Vnp[i];
            sw += coef * a.Wnp[i];
        } else {
            app += 1.5 * coef;
            su += coef * (2 * a.Unp[i] - 0.5 * a.Unp[i]);
            sv += coef * (2 * a.Vnp[i] - 0.5 * a.Vnp[i]);
            sw += coef * (2 * a.Wnp[i] - 0.5 * a.Wnp[i]);
        }
    }
    for (int s = d.cs_ptr[i]; s < d.cs_ptr[i + 1]; ++s) {
        int f = d.cs_face[s];
        if (f < d.F) {
            bool first = d.fc1[f] == i;
            double RUn = first ? a.RUFace[f] : -a.RUFace[f];
            double D = a.fD[f];
            double apn = 0.;
            if (HYB) {
                const double anb = cmax(cmax(-RUn, D - 0.5 * RUn), 0.);
                app += anb;
                apn = -anb;
            } else {
                if (RUn < 0.) {
                    apn += RUn;
                    app -= RUn;
                }
                app += D;
                apn += -D;
            }
            a.val[sell_pos(d.A, i, d.cs_k[s])] = apn;
            double e0 = a.fE[f], e1 = a.fE[d.F + f], e2 = a.fE[2 * d.F + f];
            if (first) { su += e0; sv += e1; sw += e2; }
            else { su -= e0; sv -= e1; sw -= e2; }
        } else {
            int b = f - d.F;
            app += a.bapp[b];
            su += a.bsrc[b];
            sv += a.bsrc[d.B + b];
            sw += a.bsrc[2 * d.B + b];
        }
    }
    app /= a.urf;
    a.Apr[i] = 1. / app;
    a.val[sell_pos(d.A, i, 0)] = app;
    double vol = d.vol[i];
    double U = a.U[i], V = a.V[i], W = a.W[i], R = a.R[i];
    a.bu[i] = su + (1. - a.urf) * app * U + (-a.dP[i] + R * a.g[0]) * vol;
    a.bv[i] = sv + (1. - a.urf) * app * V + (-a.dP[nc + i] + R * a.g[1]) * vol;
    a.bw[i] = sw + (1. - a.urf) * app * W + (-a.dP[2 * nc + i] + R * a.g[2]) * vol;
}

// Residual[0..2] and commit, navier_velocity.cpp:31-58
__global__ void k_commit3(DomView d, double *U, double *V, double *W, const double *x3, RedScratch rs) {
    double v[3] = {0., 0., 0.};
    const int n = d.nc;
    for (int i = blockIdx.x * NB + threadIdx.x; i < n; i += gridDim.x * NB) {
        double vol = d.vol[i];
        double x0 = x3[i], x1 = x3[n + i], x2 = x3[2 * n + i];
        v[0] += fabs(U[i] - x0) * vol;
        v[1] += fabs(V[i] - x1) * vol;
        v[2] += fabs(W[i] - x2) * vol;
        U[i] = x0; V[i] = x1; W[i] = x2;
    }
    const int slots[3] = {RED_RES0, RED_RES1, RED_RES2};
    reduce_to_slots<3>(v, slots, rs);
}

// ---------------------------------------------------------------------------
// Rhie-Chow face flux (CalRUFace2, navier_velocity.cpp:389-442) and the p'
// coupling coefficient of BuildPressureMatrix (navier_pressure.cpp:150-153).
__global__ void k_rhie_chow(DomView d, PresArgs a) {
    int f = blockIdx.x * NB + threadIdx.x;
    if (f >= d.nf) return;
    const int nc = d.nc, nf = d.nf;
    double n0 = d.fn[f], n1 = d.fn[nf + f], n2 = d.fn[2 * nf + f];
    if (f >= d.F) {
        int b = f - d.F;
        double ruf = a.BU[b] * a.BRo[b], rvf = a.BV[b] * a.BRo[b], rwf = a.BW[b] * a.BRo[b];
        a.RUFace[f] = ruf * n0 + rvf * n1 + rwf * n2;
        return;
    }
    int c1 = d.fc1[f], c2 = d.fc2[f];
    double lambda = d.flam[f];
    double lambda2 = 1. - lambda;
    double R1 = a.R[c1], R2 = a.R[c2];
    double rf = lambda * R1 + lambda2 * R2;
    double ruf = lambda * R1 * a.U[c1] + lambda2 * R2 * a.U[c2];
    double rvf = lambda * R1 * a.V[c1] + lambda2 * R2 * a.V[c2];
    double rwf = lambda * R1 * a.W[c1] + lambda2 * R2 * a.W[c2];
    double RU = ruf * n0 + rvf * n1 + rwf * n2;
    const double *xp = d.fxpac, *xn = d.fxnac;
    const int F = d.F;
    double dx0 = xp[f] - d.cx[c1], dx1 = xp[F + f] - d.cx[nc + c1], dx2 = xp[2 * F + f] - d.cx[2 * nc + c1];
    double P1 = a.P[c1] + (a.dP[c1] * dx0 + a.dP[nc + c1] * dx1 + a.dP[2 * nc + c1] * dx2);
    dx0 = xn[f] - d.cx[c2]; dx1 = xn[F + f] - d.cx[nc + c2]; dx2 = xn[2 * F + f] - d.cx[2 * nc + c2];
    double P2 = a.P[c2] + (a.dP[c2] * dx0 + a.dP[nc + c2] * dx1 + a.dP[2 * nc + c2] * dx2);
    dx0 = xn[f] - xp[f]; dx1 = xn[F + f] - xp[F + f]; dx2 = xn[2 * F + f] - xp[2 * F + f];
    double d12 = d.fd12[f];
    double Apr1 = a.Apr[c1], Apr2 = a.Apr[c2];
    double V1 = d.vol[c1], V2 = d.vol[c2];
    double aprf = lambda * Apr1 + lambda2 * Apr2;
    double vol = lambda * V1 + lambda2 * V2;
    double dpx = lambda * a.dP[c1] + lambda2 * a.dP[c2];
    double dpy = lambda * a.dP[nc + c1] + lambda2 * a.dP[nc + c2];
    double dpz = lambda * a.dP[2 * nc + c1] + lambda2 * a.dP[2 * nc + c2];
    double dpn = dpx * dx0 + dpy * dx1 + dpz * dx2;
    RU -= rf * d.farea[f] * aprf / d12 * vol * ((P2 - P1) - dpn);
    a.RUFace[f] = RU;
    double roapf = R1 * Apr1 * lambda + R2 * Apr2 * lambda2;
    double volf = V1 * lambda + V2 * lambda2;
    a.fcoef[f] = roapf * volf * d.frl[f];
}

// p' matrix rows and right-hand side, navier_pressure.cpp:88-195 (density model 0)
__global__ void k_pressure_cell(DomView d, PresArgs a) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    const bool gas = a.density_model == 1;
    double valcen = 0., bpv = 0.;
    if (gas && a.transient) valcen += -d.vol[i] / (a.dt * a.rcpcv * a.T[i]);
    for (int s = d.cs_ptr[i]; s < d.cs_ptr[i + 1]; ++s) {
        int f = d.cs_face[s];
        bool first = d.fc1[f] == i;
        double RU = a.RUFace[f];
        if (first) bpv += RU;
        else bpv -= RU;
        if (f < d.F) {
            double tmp = a.fcoef[f];
            valcen += -tmp;
            double aij = tmp;
            if (gas) {  // navier_pressure.cpp:165-181
                int in = first ? d.fc2[f] : d.fc1[f];
                double lambda = first ? d.flam[f] : 1. - d.flam[f];
                double lambda2 = 1. - lambda;
                double RUn = first ? RU : -RU;
                double rof = lambda * a.R[i] + lambda2 * a.R[in];
                if (RUn > 0.) valcen += -RUn / (rof * a.rcpcv * a.T[i]);
                if (RUn < 0.) aij += -RUn / (rof * a.rcpcv * a.T[in]);
            }
            a.val[sell_pos(d.A, i, d.cs_k[s])] = aij;
        } else if (gas) {  // navier_pressure.cpp:118-133
            int b = f - d.F;
            int type = d.btype1[b];
            if (type == 2) valcen += fmin(RU, 0.) / (a.BRo[b] * a.rcpcv * a.T[i]);
            else if (type == 3) valcen += fmax(RU, 0.) / (a.R[i] * a.rcpcv * a.T[i]);
        }
    }
    a.val[sell_pos(d.A, i, 0)] = valcen;
    a.bp[i] = bpv;
}

// navier_scalar.cpp:277-338, gathered per cell (+ for the face's cell1, - for cell2)
__global__ void k_energy_viscous(DomView d, const double *VisLam, const double *VisTur, const double *dU,
                                 const double *dV, const double *dW, const double *U, const double *V,
                                 const double *W, double cp, double *src) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    const int nc = d.nc, nf = d.nf;
    double acc = src[i];
    for (int s = d.cs_ptr[i]; s < d.cs_ptr[i + 1]; ++s) {
        int f = d.cs_face[s];
        int c1 = d.fc1[f], c2 = d.fc2[f];
        double VisL, VisT, g[9], vx, vy, vz;
        const double *gr[3] = {dU, dV, dW};
        if (c2 < 0) {
            VisL = VisLam[c1];
            VisT = VisTur[c1];
            for (int q = 0; q < 3; ++q)
                for (int k = 0; k < 3; ++k) g[3 * q + k] = gr[q][(size_t)k * nc + c1];
            vx = U[c1];
            vy = V[c1];
            vz = W[c1];
        } else {
            double lambda = d.flam[f], lambda2 = 1. - lambda;
            VisL = lambda * VisLam[c1] + lambda2 * VisLam[c2];
            VisT = lambda * VisTur[c1] + lambda2 * VisTur[c2];
            for (int q = 0; q < 3; ++q)
                for (int k = 0; k < 3; ++k)
                    g[3 * q + k] = lambda * gr[q][(size_t)k * nc + c1] + lambda2 * gr[q][(size_t)k * nc + c2];
            vx = lambda * U[c1] + lambda2 * U[c2];
            vy = lambda * V[c1] + lambda2 * V[c2];
            vz = lambda * W[c1] + lambda2 * W[c2];
        }
        double dudx = g[0], dudy = g[1], dudz = g[2], dvdx = g[3], dvdy = g[4], dvdz = g[5];
        double dwdx = g[6], dwdy = g[7], dwdz = g[8];
        double vmul = VisL + VisT;
        double vlac = -2. / 3. * vmul;
        double div = dudx + dvdy + dwdz;
        double txx = 2. * vmul * dudx + vlac * div;
        double tyy = 2. * vmul * dvdy + vlac * div;
        double tzz = 2. * vmul * dwdz + vlac * div;
        double txy = vmul * (dudy + dvdx);
        double txz = vmul * (dudz + dwdx);
        double tyz = vmul * (dvdz + dwdy);
        double btx = vx * txx + vy * txy + vz * txz;
        double bty = vx * txy + vy * tyy + vz * tyz;
        double btz = vx * txz + vy * tyz + vz * tzz;
        double fvis = (btx * d.fn[f] + bty * d.fn[nf + f] + btz * d.fn[2 * nf + f]) / cp;
        acc += (c1 == i) ? fvis : -fvis;
    }
    src[i] = acc;
}

// navier_pressure.cpp:38-56
__global__ void k_correct_cells(DomView d, CorrArgs a, RedScratch rs) {
    double v[1] = {0.};
    const int n = d.nc;
    double dpref = a.dp[a.cell_ref];
    for (int i = blockIdx.x * NB + threadIdx.x; i < n; i += gridDim.x * NB) {
        double dpi = a.dp[i];
        double vol = d.vol[i];
        v[0] += fabs(dpi - dpref) * vol;
        if (a.density_model == 1) {  // navier_pressure.cpp:45-48
            a.P[i] = a.P[i] + a.urf_p * dpi;
            a.R[i] += dpi / (a.rcpcv * a.T[i]);
        } else {
            a.P[i] = a.P[i] + a.urf_p * (dpi - dpref);
        }
        double coef = vol * a.Apr[i];
        a.U[i] = a.U[i] - coef * a.dPdp[i];
        a.V[i] = a.V[i] - coef * a.dPdp[n + i];
        a.W[i] = a.W[i] - coef * a.dPdp[2 * n + i];
    }
    const int slots[1] = {RED_RES3};
    reduce_to_slots<1>(v, slots, rs);
}

// CorrectRUFace2, navier_pressure.cpp:200-242
__global__ void k_correct_faces(DomView d, const double *dp, const double *dPdp, const double *R,
                                const double *Apr, const double *BRo, const double *BU, const double *BV,
                                const double *BW, double urf_p, double *RUFace, const double *fcoef,
                                int density_model, const double *T, double rcpcv) {
    int f = blockIdx.x * NB + threadIdx.x;
    if (f >= d.nf) return;
    const int nc = d.nc, nf = d.nf, F = d.F;
    if (f >= F) {
        int b = f - F;
        double ruf = BU[b] * BRo[b], rvf = BV[b] * BRo[b], rwf = BW[b] * BRo[b];
        RUFace[f] = ruf * d.fn[f] + rvf * d.fn[nf + f] + rwf * d.fn[2 * nf + f];
        return;
    }
    int c1 = d.fc1[f], c2 = d.fc2[f];
    double dx10 = d.fxpac[f] - d.cx[c1], dx11 = d.fxpac[F + f] - d.cx[nc + c1],
           dx12 = d.fxpac[2 * F + f] - d.cx[2 * nc + c1];
    double dx20 = d.fxnac[f] - d.cx[c2], dx21 = d.fxnac[F + f] - d.cx[nc + c2],
           dx22 = d.fxnac[2 * F + f] - d.cx[2 * nc + c2];
    double coef = fcoef[f];
    if (density_model == 1) {  // rho' u, and rho Apr from the corrected density
        double lambda = d.flam[f], lambda2 = 1. - lambda;
        double rop = dp[c1] / (rcpcv * T[c1]) * lambda + dp[c2] / (rcpcv * T[c2]) * lambda2;
        double rof = R[c1] * lambda + R[c2] * lambda2;
        RUFace[f] += RUFace[f] * rop / rof;
        double roapf = R[c1] * Apr[c1] * lambda + R[c2] * Apr[c2] * lambda2;
        double vol = d.vol[c1] * lambda + d.vol[c2] * lambda2;
        coef = roapf * vol * d.frl[f];
    }
    double dp1 = dp[c1] + urf_p * (dPdp[c1] * dx10 + dPdp[nc + c1] * dx11 + dPdp[2 * nc + c1] * dx12);
    double dp2 = dp[c2] + urf_p * (dPdp[c2] * dx20 + dPdp[nc + c2] * dx21 + dPdp[2 * nc + c2] * dx22);
    RUFace[f] += -coef * (dp2 - dp1);
}

// ---------------------------------------------------------------------------
// Scalar transport assembly.  Fluid: navier_scalar.cpp:466-647 (+ the energy
// wall callback :176-248); solid: HeatConductionSolver.cpp:175-288.
template <bool HYB>
__global__ void k_scalar_face(DomView d, ScalarArgs a) {
    int f = blockIdx.x * NB + threadIdx.x;
    if (f >= d.F) return;
    const int nc = d.nc, nf = d.nf;
    int c1 = d.fc1[f], c2 = d.fc2[f];
    double lambda = d.flam[f];
    double lambda2 = 1. - lambda;
    double sav1 = d.fn[f], sav2 = d.fn[nf + f], sav3 = d.fn[2 * nf + f];
    double Visc = lambda * a.diff[c1] + lambda2 * a.diff[c2];
    double gx = lambda * a.grad[c1] + lambda2 * a.grad[c2];
    double gy = lambda * a.grad[nc + c1] + lambda2 * a.grad[nc + c2];
    double gz = lambda * a.grad[2 * nc + c1] + lambda2 * a.grad[2 * nc + c2];
    double D = Visc * d.frl[f];
    double fcs = 0.;
    if (a.bc_mode != SC_SOLID && !HYB) {
        double RU = a.RUFace[f];
        int up = RU > 0. ? c1 : c2;
        double dx0 = d.fx[f] - d.cx[up], dx1 = d.fx[nf + f] - d.cx[nc + up], dx2 = d.fx[2 * nf + f] - d.cx[2 * nc + up];
        double pfi = a.phi[up];
        double pfh = pfi + (a.grad[up] * dx0 + a.grad[nc + up] * dx1 + a.grad[2 * nc + up] * dx2);
        fcs = RU * (pfh - pfi);
    }
    double fde = Visc * (gx * sav1 + gy * sav2 + gz * sav3);
    double dxc0 = d.cx[c2] - d.cx[c1], dxc1 = d.cx[nc + c2] - d.cx[nc + c1], dxc2 = d.cx[2 * nc + c2] - d.cx[2 * nc + c1];
    double fdi = D * (gx * dxc0 + gy * dxc1 + gz * dxc2);
    a.fD[f] = D;
    a.fE[f] = fde - fdi - fcs;
}

__global__ void k_scalar_bnd(DomView d, ScalarArgs a) {
    int b = blockIdx.x * NB + threadIdx.x;
    if (b >= d.B) return;
    const int nc = d.nc, nf = d.nf;
    int i = d.bcell[b];
    int f = d.F + b;
    int t1 = d.btype1[b], t2 = d.btype2[b];
    double sav1 = d.fn[f], sav2 = d.fn[nf + f], sav3 = d.fn[2 * nf + f];
    double Visc = a.diff[i];
    double gx = a.grad[i], gy = a.grad[nc + i], gz = a.grad[2 * nc + i];
    double dxc0 = d.fx[f] - d.cx[i], dxc1 = d.fx[nf + f] - d.cx[nc + i], dxc2 = d.fx[2 * nf + f] - d.cx[2 * nc + i];
    double app = 0., fde = 0., fdi = 0., fcs = 0.;
    bool dirichlet;
    if (a.bc_mode == SC_SOLID) {
        if (t1 == 1 && t2 == 0) dirichlet = true;
        else if (t1 == 1 || t1 == 4) {
            dirichlet = false;
            fde = 0. - a.Bq[b] * d.farea[f];
        } else {
            dirichlet = false;
            atomicOr(a.flags, 1);
        }
    } else if (a.bc_mode == SC_FLUID_ENERGY) {
        if (t1 == 1 && t2 == 1) {
            dirichlet = false;
            fde = 0. - a.Bq[b] * d.farea[f];
        } else if (t1 == 4) {
            dirichlet = false;
        } else {
            dirichlet = true;
        }
    } else {
        dirichlet = (t1 >= 1 && t1 <= 4);
        if (!dirichlet) atomicOr(a.flags, 1);
    }
    if (dirichlet) {
        double VAL = Visc * d.frl[f];
        app += VAL;
        fde = Visc * (gx * sav1 + gy * sav2 + gz * sav3);
        fdi = VAL * (gx * dxc0 + gy * dxc1 + gz * dxc2 - a.Bphi[b]);
    }
    if (a.bc_mode != SC_SOLID && (t1 == 2 || t1 == 3)) {
        double RU = a.RUFace[f];
        if (t1 == 2 && RU > 0) atomicOr(a.flags, 2);  // reverse flow out of an inlet: the reference stops
        double fl = cmin(RU, 0.0);
        app -= fl;
        fcs = fl * a.Bphi[b];
    }
    a.bapp[b] = app;
    a.bsrc[b] = fde - fdi - fcs;
}

template <bool HYB>
__global__ void k_scalar_cell(DomView d, ScalarArgs a) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    double app = a.app0[i];
    double sphi = a.src[i];
    bool conv = a.bc_mode != SC_SOLID;
    for (int s = d.cs_ptr[i]; s < d.cs_ptr[i + 1]; ++s) {
        int f = d.cs_face[s];
        if (f < d.F) {
            bool first = d.fc1[f] == i;
            double apn = 0.;
            double D = a.fD[f];
            if (conv && HYB) {
                const double RUn = first ? a.RUFace[f] : -a.RUFace[f];
                const double anb = cmax(cmax(-RUn, D - 0.5 * RUn), 0.);
                app += anb;
                apn = -anb;
            } else {
                if (conv) {
                    double RUn = first ? a.RUFace[f] : -a.RUFace[f];
                    if (RUn < 0.) {
                        apn += RUn;
                        app -= RUn;
                    }
                }
                app += D;
                apn += -D;
            }
            a.val[sell_pos(d.A, i, d.cs_k[s])] = apn;
            double e = a.fE[f];
            if (first) sphi += e;
            else sphi -= e;
        } else {
            int b = f - d.F;
            app += a.bapp[b];
            sphi += a.bsrc[b];
        }
    }
    app /= a.urf;
    a.val[sell_pos(d.A, i, 0)] = app;
    a.b[i] = sphi + (1. - a.urf) * app * a.phi[i];
}

// ---------------------------------------------------------------------------
// k-epsilon, navier_scalar.cpp:36-67 and the wall functions of
// navier_bc.cpp:229-278 (applied per cell, in boundary-record order).
namespace ke {
constexpr double kappa = 0.419, Cmu = 0.09, Ceps1 = 1.44, Ceps2 = 1.92, Sigma_k = 1.0, Sigma_e = 1.3;
}

__global__ void k_ke_sources(DomView d, KeArgs a) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    const int nc = d.nc, nf = d.nf;
    double vol = d.vol[i];
    a.VisTE[i] = a.VisLam[i] + a.VisTur[i] / ke::Sigma_k;
    a.VisED[i] = a.VisLam[i] + a.VisTur[i] / ke::Sigma_e;
    double du0 = a.dU[i], du1 = a.dU[nc + i], du2 = a.dU[2 * nc + i];
    double dv0 = a.dV[i], dv1 = a.dV[nc + i], dv2 = a.dV[2 * nc + i];
    double dw0 = a.dW[i], dw1 = a.dW[nc + i], dw2 = a.dW[2 * nc + i];
    double s1 = (du0 + du0) * du0 + (du1 + dv0) * du1 + (du2 + dw0) * du2;
    double s2 = (dv0 + du1) * dv0 + (dv1 + dv1) * dv1 + (dv2 + dw1) * dv2;
    double s3 = (dw0 + du2) * dw0 + (dw1 + dv2) * dw1 + (dw2 + dw2) * dw2;
    double prod = a.VisTur[i] * (s1 + s2 + s3);
    double R = a.R[i];
    double TE = a.TE[i], ED = a.ED[i];
    double Dis = R * ED;
    double tesrc = prod * vol;
    double apte = Dis / TE * vol;
    for (int k = d.cw_ptr[i]; k < d.cw_ptr[i + 1]; ++k) {
        int b = d.cw_b[k];
        int f = d.F + b;
        a.BTE[b] = TE;
        a.BED[b] = ED;
        double area = d.farea[f];
        double sav1n = d.fn[f] / (area + 1.e-16), sav2n = d.fn[nf + f] / (area + 1.e-16),
               sav3n = d.fn[2 * nf + f] / (area + 1.e-16);
        double U = a.U[i], V = a.V[i], W = a.W[i];
        double vnor = U * sav1n + V * sav2n + W * sav3n;
        double vt1 = U - vnor * sav1n, vt2 = V - vnor * sav2n, vt3 = W - vnor * sav3n;
        double vel = sqrt(vt1 * vt1 + vt2 * vt2 + vt3 * vt3);
        double dist = d.bdist[b];
        double Cmu25 = pow(ke::Cmu, 0.25);
        double utau = Cmu25 * sqrt(TE);
        double yplus = dist * utau * R / (a.VisLam[i] + SMALL);
        double tauw = a.VisLam[i] * vel / dist;
        if (yplus < 11.) utau = sqrt(tauw / R);
        else utau = Cmu25 * sqrt(TE);
        prod = tauw * utau / (ke::kappa * dist);
        double eps = pow(ke::Cmu, 0.75) * pow(TE, 1.5) / (ke::kappa * dist);
        tesrc = prod * vol;
        apte -= R * ED / TE * vol;
        apte += R * eps / TE * vol;
        ED = eps;
        a.BED[b] = eps;
    }
    a.Prod[i] = prod;
    a.TESrc[i] = tesrc;
    a.ApTE[i] = apte;
    a.EDSrc[i] = 0.;
    a.ApED[i] = 0.;
    a.ED[i] = ED;
}

// inlet / outlet / symmetry values of k and epsilon, navier_bc.cpp:520-555
// (these loops test the region id against 2/3/4)
__global__ void k_ke_bnd(DomView d, KeArgs a) {
    int b = blockIdx.x * NB + threadIdx.x;
    if (b >= d.B) return;
    int rid = d.brid[b];
    int ic = d.bcell[b];
    if (rid == 2) {
        a.BTE[b] = d.bin[6 * d.B + b];
        a.BED[b] = d.bin[7 * d.B + b];
    } else if (rid == 3 || rid == 4) {
        a.BTE[b] = a.TE[ic];
        a.BED[b] = a.ED[ic];
    }
}

// navier_scalar.cpp:116-122
__global__ void k_ke_eps_src(DomView d, KeArgs a) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc) return;
    double fact = a.ED[i] / (a.TE[i] + SMALL) * d.vol[i];
    a.EDSrc[i] = ke::Ceps1 * fact * a.Prod[i];
    a.ApED[i] += ke::Ceps2 * fact * a.R[i];
}

// navier_scalar.cpp:130-139: wall cells get the row "eps = eps_wall"
__global__ void k_ke_eps_rows(DomView d, const double *ED, double *val, double *b) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= d.nc || d.cw_ptr[i] == d.cw_ptr[i + 1]) return;
    int w = d.A.sl_w[i >> 5];
    for (int k = 1; k < w; ++k) val[sell_pos(d.A, i, k)] = 0.;
    val[sell_pos(d.A, i, 0)] = 1.;
    b[i] = ED[i];
}

__global__ void k_clip_max(double *dst, const double *src, double lo, int n) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i < n) dst[i] = cmax(lo, src[i]);
}

__global__ void k_visc_tur(int n, const double *R, const double *TE, const double *ED, double *VisTur) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= n) return;
    double ed = ED[i], te = TE[i];
    VisTur[i] = (ed > 1.e-12) ? ke::Cmu * R[i] * te * te / (ed + SMALL) : 0.;
}

// ---------------------------------------------------------------------------
// energy
__global__ void k_kcond(int n, const double *VisLam, const double *VisTur, double cp, double prl, double prte,
                        double *kcond) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= n) return;
    double k = cp * (VisLam[i] / prl + VisTur[i] / prte) / cp;
    kcond[i] = k * 100;  // navier_scalar.cpp:272
}

__global__ void k_bc_temp_fluid(DomView d, const double *T, double *BTem) {
    int b = blockIdx.x * NB + threadIdx.x;
    if (b >= d.B) return;
    int t1 = d.btype1[b], t2 = d.btype2[b];
    int ic = d.bcell[b];
    if ((t1 == 1 && t2 == 1) || t1 == 3 || t1 == 4) BTem[b] = T[ic];
}

__global__ void k_bc_temp_solid(DomView d, const double *T, const double *diff, const double *Bq, double *BTem) {
    int b = blockIdx.x * NB + threadIdx.x;
    if (b >= d.B) return;
    int t1 = d.btype1[b], t2 = d.btype2[b];
    int ic = d.bcell[b];
    int f = d.F + b;
    if (t1 == 1 && t2 == 1) BTem[b] = T[ic] - Bq[b] / (diff[ic] * d.frl[f]);
    else if ((t1 == 1 && t2 == 2) || t1 == 4) BTem[b] = T[ic];
}

__global__ void k_cht_s2f(DomView s, const double *Ts, const double *gTs, DomView fl, double *BTem_f) {
    int k = blockIdx.x * NB + threadIdx.x;
    int ncpl = s.B - s.ncb;
    if (k >= ncpl) return;
    int sb = s.ncb + k;
    int icell = s.bcell[sb];
    int f = s.F + sb;
    const int n = s.nc, nf = s.nf;
    double dx0 = s.fx[f] - s.cx[icell], dx1 = s.fx[nf + f] - s.cx[n + icell], dx2 = s.fx[2 * nf + f] - s.cx[2 * n + icell];
    double dtdr = gTs[icell] * dx0 + gTs[n + icell] * dx1 + gTs[2 * n + icell] * dx2;
    BTem_f[fl.ncb + k] = Ts[icell] + dtdr;
}

__global__ void k_cht_f2s(DomView fl, const double *gTf, const double *kcond, double *Bq_f, DomView s, double *Bq_s) {
    int k = blockIdx.x * NB + threadIdx.x;
    int ncpl = fl.B - fl.ncb;
    if (k >= ncpl) return;
    int fb = fl.ncb + k;
    int fc = fl.bcell[fb];
    int f = fl.F + fb;
    const int n = fl.nc, nf = fl.nf;
    double dtdn = (gTf[fc] * fl.fn[f] + gTf[n + fc] * fl.fn[nf + f] + gTf[2 * n + fc] * fl.fn[2 * nf + f]) / fl.farea[f];
    double q = 0. - dtdn * kcond[fc];
    Bq_f[fb] = q;
    Bq_s[s.ncb + k] = 0. - q;
}

__global__ void k_time_term(int n, const double *R, const double *vol, double dt, int scheme, const double *old,
                            double *app, double *src) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i >= n) return;
    double coef = R[i] / dt * vol[i];
    if (scheme == 1) {
        app[i] += coef;
        src[i] += coef * old[i];
    } else {
        app[i] += 1.5 * coef;
        src[i] += coef * (2 * old[i] - 0.5 * old[i]);
    }
}

__global__ void k_fill(double *x, double v, int n) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i < n) x[i] = v;
}
__global__ void k_copy(double *dst, const double *src, int n) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i < n) dst[i] = src[i];
}
__global__ void k_scale_src(double *dst, const double *vol, double q, int n) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i < n) dst[i] = q * vol[i];
}

__global__ void k_gather(double *dst, const double *src, const int *idx, int n) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}
__global__ void k_scatter(double *dst, const double *src, const int *idx, int n) {
    int i = blockIdx.x * NB + threadIdx.x;
    if (i < n) dst[idx[i]] = src[i];
}
__global__ void k_aos3_to_soa3(double *dst, const double *src, int n) {
    int t = blockIdx.x * NB + threadIdx.x;
    if (t >= 3 * n) return;
    int i = t / 3, k = t % 3;
    dst[(size_t)k * n + i] = src[t];
}
__global__ void k_soa3_to_aos3(double *dst, const double *src, int n) {
    int t = blockIdx.x * NB + threadIdx.x;
    if (t >= 3 * n) return;
    int i = t / 3, k = t % 3;
    dst[t] = src[(size_t)k * n + i];
}

#define CHECK_LAUNCH() SYSU_CUDA(cudaGetLastError())

}  // namespace

// ===========================================================================
void red_reset(RedScratch rs, cudaStream_t st) {
    SYSU_CUDA(cudaMemsetAsync(rs.out, 0, RED_NSLOT * sizeof(double), st));
    SYSU_CUDA(cudaMemsetAsync(rs.ticket, 0, sizeof(unsigned int), st));
}

void launch_bc_velocity(const DomView &d, const double *R, const double *U, const double *V, const double *W,
                        double *BRo, double *BU, double *BV, double *BW, bool has_outlet, RedScratch rs,
                        cudaStream_t st) {
    if (d.B == 0) return;
    { k_bc_velocity<<<nblk_capped(d.B, rs.max_blocks), NB, 0, st>>>(d, R, U, V, W, BRo, BU, BV, BW, has_outlet ? 1 : 0, rs); ++::sysu::g_launches; }
    CHECK_LAUNCH();
    if (has_outlet) {
        { k_bc_outlet<<<nblk(d.B), NB, 0, st>>>(d, BU, BV, BW, rs.out); ++::sysu::g_launches; }
        CHECK_LAUNCH();
    }
}

void launch_gradient(const DomView &d, int nfield, const double *const *phi, const double *const *Bphi,
                     double *const *grad, cudaStream_t st) {
    GradPtrs p{};
    for (int k = 0; k < nfield; ++k) {
        p.phi[k] = phi[k];
        p.Bphi[k] = Bphi[k];
        p.grad[k] = grad[k];
    }
    if (nfield != 1 && nfield != 3 && nfield != 4) throw CaseError{"launch_gradient: 1, 3 or 4 fields"};
    if (d.lsq_c) {
        switch (nfield) {
        case 1: k_gradient_lsq<1><<<nblk(d.nc), NB, 0, st>>>(d, p); break;
        case 3: k_gradient_lsq<3><<<nblk(d.nc), NB, 0, st>>>(d, p); break;
        default: k_gradient_lsq<4><<<nblk(d.nc), NB, 0, st>>>(d, p); break;
        }
    } else {
        switch (nfield) {
        case 1: k_gradient_v<1><<<nblk(d.nc), NB, 0, st>>>(d, p); break;
        case 3: k_gradient_v<3><<<nblk(d.nc), NB, 0, st>>>(d, p); break;
        default: k_gradient_v<4><<<nblk(d.nc), NB, 0, st>>>(d, p); break;
        }
    }
    ++::sysu::g_launches;
    CHECK_LAUNCH();
}

void launch_lsq_setup(const DomView &d, double *lsq_c, cudaStream_t st) {
    if (d.nc == 0) return;
    { k_lsq_setup<<<nblk(d.nc), NB, 0, st>>>(d, lsq_c); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_limiter(const DomView &d, int limiter, const double *phi, double *grad, double *tmp3,
                    double *tmp_v, cudaStream_t st) {
    if (limiter == 0) return;
    if (limiter == 3) {
        { k_limiter_weno<<<nblk(d.nc), NB, 0, st>>>(d, grad, tmp3); ++::sysu::g_launches; }
        { k_copy3<<<nblk(3 * d.nc), NB, 0, st>>>(d.nc, tmp3, grad); ++::sysu::g_launches; }
    } else if (limiter == 1) {
        { k_limiter_barth<<<nblk(d.nc), NB, 0, st>>>(d, phi, grad); ++::sysu::g_launches; }
    } else if (limiter == 2) {
        { k_vertex_minmax<<<nblk(d.nv), NB, 0, st>>>(d, phi, tmp_v, tmp_v + d.nv); ++::sysu::g_launches; }
        { k_limiter_mlp<<<nblk(d.nc), NB, 0, st>>>(d, phi, tmp_v, tmp_v + d.nv, grad); ++::sysu::g_launches; }
    } else {
        throw CaseError{"no such limiter choice"};
    }
    CHECK_LAUNCH();
}

void launch_momentum(const DomView &d, const MomArgs &a, cudaStream_t st) {
    if (d.F) {
        if (a.hybrid) k_mom_face<true><<<nblk(d.F), NB, 0, st>>>(d, a);
        else k_mom_face<false><<<nblk(d.F), NB, 0, st>>>(d, a);
        ++::sysu::g_launches;
    }
    if (d.B) { k_mom_bnd<<<nblk(d.B), NB, 0, st>>>(d, a); ++::sysu::g_launches; }
    if (a.hybrid) k_mom_cell<true><<<nblk(d.nc), NB, 0, st>>>(d, a);
    else k_mom_cell<false><<<nblk(d.nc), NB, 0, st>>>(d, a);
    ++::sysu::g_launches;
    CHECK_LAUNCH();
}

void launch_commit3(const DomView &d, double *U, double *V, double *W, const double *x3, RedScratch rs,
                    cudaStream_t st) {
    { k_commit3<<<nblk_capped(d.nc, rs.max_blocks), NB, 0, st>>>(d, U, V, W, x3, rs); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_gather(double *dst, const double *src, const int *idx, int n, cudaStream_t st) {
    if (n <= 0) return;
    { k_gather<<<nblk(n), NB, 0, st>>>(dst, src, idx, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_scatter(double *dst, const double *src, const int *idx, int n, cudaStream_t st) {
    if (n <= 0) return;
    { k_scatter<<<nblk(n), NB, 0, st>>>(dst, src, idx, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_aos3_to_soa3(double *dst, const double *src, int n, cudaStream_t st) {
    if (n <= 0) return;
    { k_aos3_to_soa3<<<nblk(3 * n), NB, 0, st>>>(dst, src, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_soa3_to_aos3(double *dst, const double *src, int n, cudaStream_t st) {
    if (n <= 0) return;
    { k_soa3_to_aos3<<<nblk(3 * n), NB, 0, st>>>(dst, src, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_energy_viscous(const DomView &d, const double *VisLam, const double *VisTur, const double *dU,
                           const double *dV, const double *dW, const double *U, const double *V, const double *W,
                           double cp, double *src, cudaStream_t st) {
    if (d.nc == 0) return;
    { k_energy_viscous<<<nblk(d.nc), NB, 0, st>>>(d, VisLam, VisTur, dU, dV, dW, U, V, W, cp, src); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_pressure_assembly(const DomView &d, const PresArgs &a, cudaStream_t st) {
    { k_rhie_chow<<<nblk(d.nf), NB, 0, st>>>(d, a); ++::sysu::g_launches; }
    { k_pressure_cell<<<nblk(d.nc), NB, 0, st>>>(d, a); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_correct_cells(const DomView &d, const CorrArgs &a, RedScratch rs, cudaStream_t st) {
    { k_correct_cells<<<nblk_capped(d.nc, rs.max_blocks), NB, 0, st>>>(d, a, rs); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_correct_faces(const DomView &d, const double *dp, const double *dPdp, const double *R,
                          const double *Apr, const double *BRo, const double *BU, const double *BV,
                          const double *BW, double urf_p, double *RUFace, const double *fcoef, int density_model,
                          const double *T, double rcpcv, cudaStream_t st) {
    { k_correct_faces<<<nblk(d.nf), NB, 0, st>>>(d, dp, dPdp, R, Apr, BRo, BU, BV, BW, urf_p, RUFace, fcoef, density_model, T, rcpcv); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_scalar(const DomView &d, const ScalarArgs &a, cudaStream_t st) {
    if (d.F) {
        if (a.hybrid) k_scalar_face<true><<<nblk(d.F), NB, 0, st>>>(d, a);
        else k_scalar_face<false><<<nblk(d.F), NB, 0, st>>>(d, a);
        ++::sysu::g_launches;
    }
    if (d.B) { k_scalar_bnd<<<nblk(d.B), NB, 0, st>>>(d, a); ++::sysu::g_launches; }
    if (a.hybrid) k_scalar_cell<true><<<nblk(d.nc), NB, 0, st>>>(d, a);
    else k_scalar_cell<false><<<nblk(d.nc), NB, 0, st>>>(d, a);
    ++::sysu::g_launches;
    CHECK_LAUNCH();
}

void launch_ke_sources(const DomView &d, const KeArgs &a, cudaStream_t st) {
    { k_ke_sources<<<nblk(d.nc), NB, 0, st>>>(d, a); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_ke_bnd_values(const DomView &d, const KeArgs &a, cudaStream_t st) {
    if (!d.B) return;
    { k_ke_bnd<<<nblk(d.B), NB, 0, st>>>(d, a); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_ke_eps_sources(const DomView &d, const KeArgs &a, cudaStream_t st) {
    { k_ke_eps_src<<<nblk(d.nc), NB, 0, st>>>(d, a); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_ke_eps_wall_rows(const DomView &d, const double *ED, double *val, double *b, cudaStream_t st) {
    { k_ke_eps_rows<<<nblk(d.nc), NB, 0, st>>>(d, ED, val, b); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_clip_max(double *dst, const double *src, double lo, int n, cudaStream_t st) {
    { k_clip_max<<<nblk(n), NB, 0, st>>>(dst, src, lo, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_visc_tur(int n, const double *R, const double *TE, const double *ED, double *VisTur, cudaStream_t st) {
    { k_visc_tur<<<nblk(n), NB, 0, st>>>(n, R, TE, ED, VisTur); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_kcond(int n, const double *VisLam, const double *VisTur, double cp, double prl, double prte,
                  double *kcond, cudaStream_t st) {
    { k_kcond<<<nblk(n), NB, 0, st>>>(n, VisLam, VisTur, cp, prl, prte, kcond); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_bc_temperature_fluid(const DomView &d, const double *T, double *BTem, cudaStream_t st) {
    if (!d.B) return;
    { k_bc_temp_fluid<<<nblk(d.B), NB, 0, st>>>(d, T, BTem); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_bc_temperature_solid(const DomView &d, const double *T, const double *diff, const double *Bq,
                                 double *BTem, cudaStream_t st) {
    if (!d.B) return;
    { k_bc_temp_solid<<<nblk(d.B), NB, 0, st>>>(d, T, diff, Bq, BTem); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_cht_solid2fluid(const DomView &s, const double *Ts, const double *gTs, const DomView &f,
                            double *BTem_f, cudaStream_t st) {
    int n = s.B - s.ncb;
    if (n <= 0) return;
    { k_cht_s2f<<<nblk(n), NB, 0, st>>>(s, Ts, gTs, f, BTem_f); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_cht_fluid2solid(const DomView &f, const double *gTf, const double *kcond, double *Bq_f,
                            const DomView &s, double *Bq_s, cudaStream_t st) {
    int n = f.B - f.ncb;
    if (n <= 0) return;
    { k_cht_f2s<<<nblk(n), NB, 0, st>>>(f, gTf, kcond, Bq_f, s, Bq_s); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_time_term(int n, const double *R, const double *vol, double dt, int scheme, const double *old,
                      double *app, double *src, cudaStream_t st) {
    if (n <= 0 || scheme == 0) return;
    { k_time_term<<<nblk(n), NB, 0, st>>>(n, R, vol, dt, scheme, old, app, src); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

void launch_fill(double *x, double v, int n, cudaStream_t st) {
    if (n <= 0) return;
    { k_fill<<<nblk(n), NB, 0, st>>>(x, v, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_copy(double *dst, const double *src, int n, cudaStream_t st) {
    if (n <= 0) return;
    { k_copy<<<nblk(n), NB, 0, st>>>(dst, src, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_scale_src(double *dst, const double *vol, double q, int n, cudaStream_t st) {
    if (n <= 0) return;
    { k_scale_src<<<nblk(n), NB, 0, st>>>(dst, vol, q, n); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}
void launch_bnd_from_cell(const DomView &d, const double *phi, double *Bphi, cudaStream_t st) {
    if (!d.B) return;
    { k_bnd_from_cell<<<nblk(d.B), NB, 0, st>>>(d, phi, Bphi); ++::sysu::g_launches; }
    CHECK_LAUNCH();
}

}  // namespace sysu
