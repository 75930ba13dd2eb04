// conv_faces.cuh -- the per-face arithmetic of convdiff (6_convdiff.f90:14-167)
// with classico der = 3 (7_advectivo.f90:171-284) and the fused terms of
// complementos (11_diversos.f90:355-450), written once over an accessor so
// that the kernel that gathers its operands from global memory and the one
// that reads them from TMA-staged shared memory run the same operations.
//
// An accessor A provides u, v, w, mu, rho, xmu, ymu, zmu (a, b, c) -> T for
// box indices (a, b, c) of the case (the reference's indices, ghosts
// included).  The face functions return F before the complementos terms.
// IN = true states that the position is interior -- 2 <= i <= nx - 1,
// 2 <= j <= ny - 1, 2 <= k <= nz - 1 -- where every boundary branch of the
// stencils takes its interior case; the operations are the same.  VZ = true
// is SuLi-ICdz's variable z spacing (c.dzk set): its z interpolations
// weighted by the spacing and its z differences over dz(k) or dzz(k), as
// SuLi-ICdz/6_convdiff.f90:75-176 and 7_advectivo.f90:175-250 have them.
#pragma once

#include "suli_kernels.cuh"

namespace suli {

// interp?_cf at face f (1..n+1) of a centre quantity get(m), m in 1..n
// (8_derivadas.f90:305-479); `periodic` only for x (interpx_cf).
template <typename T, bool IN = false, typename F>
__device__ __forceinline__ T interp_cf(int f, int n, bool periodic, F get)
{
    if (IN || (f >= 2 && f <= n)) return (get(f) + get(f - 1)) * T(0.5);
    if (periodic) return (get(1) + get(n)) * T(0.5);
    if (f == 1) return (get(2) + get(1)) * T(0.5);
    return (get(n) + get(n - 1)) * T(0.5);
}

__device__ __forceinline__ int clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }
template <bool IN> __device__ __forceinline__ int clampi_in(int a, int lo, int hi) { return IN ? a : clampi(a, lo, hi); }

template <typename T>
__device__ __forceinline__ T upw(T vel, T dneg, T dpos)
{
    T a1 = vel > T(0.) ? vel : T(0.);
    T a2 = vel < T(0.) ? vel : T(0.);
    return a1 * dneg + a2 * dpos;
}

// derivaxu2n / derivaxu2p etc. (8_derivadas.f90:75-300) on a haloed array
// whose interior extent along the axis is `dim`.
// (divisions by the fixed spacing are multiplications by its reciprocal rh;
// GB300's FP64 divide is a long instruction sequence)
template <typename T, bool IN = false, typename F>
__device__ __forceinline__ T d2n(int m, int dim, bool perx, T rh, F a)
{
    if (IN || m >= 2) return T(0.5) * (a(m - 2) - 4 * a(m - 1) + 3 * a(m)) * rh;
    if (!perx) return T(0.5) * (a(m + 1) - a(m - 1)) * rh;
    return T(0.5) * (a(dim - 1) - 4 * a(dim) + 3 * a(m)) * rh;
}
template <typename T, bool IN = false, typename F>
__device__ __forceinline__ T d2p(int m, int dim, bool perx, T rh, F a)
{
    if (IN || m <= dim - 1) return T(0.5) * (-a(m + 2) + 4 * a(m + 1) - 3 * a(m)) * rh;
    if (!perx) return T(0.5) * (a(m + 1) - a(m - 1)) * rh;
    return T(0.5) * (-a(2) + 4 * a(1) - 3 * a(m)) * rh;
}

// surface tension (t_tens = 1): sigma times the face value of hs_a kurv / rho
// on the axis-0/1/2 face (i, j, k) (11_diversos.f90:383-390; interpx_cf wraps
// on a periodic x, interpy_cf / interpz_cf never wrap)
template <typename T>
__device__ __forceinline__ T tension_face(const CaseDev<T> &c, int axis, int i, int j, int k)
{
    const Geo &g = c.g;
    auto v = [&](const T *hs, long long q) { return hs[q] * c.kurv[q] / c.rho[q]; };
    T f;
    if (axis == 0) f = interp_cf<T>(i, g.nx, c.ccx0 == 0, [&](int m) { return v(c.hsx, g.at(m, j, k)); });
    else if (axis == 1) f = interp_cf<T>(j, g.ny, false, [&](int m) { return v(c.hsy, g.at(i, m, k)); });
    else f = interp_cf<T>(k, g.nz, false, [&](int m) { return v(c.hsz, g.at(i, j, m)); });
    return T(c.sigma) * f;
}

// the kinetic-energy term of complementos (m_turb >= 2, 11_diversos.f90:403-444):
// 2/3 (karho(m) - karho(m-1)) / (h rho_face) on the axis-0/1/2 face (i, j, k),
// karho = ka rhof with rhof = fantasmas_cf(rho) (8_derivadas.f90:625-671: y and
// z ghosts copy the adjacent cell, x ghosts wrap on a periodic x)
template <typename T>
__device__ __forceinline__ T ka_face(const CaseDev<T> &c, int axis, int i, int j, int k)
{
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool per = (c.ccx0 == 0);
    auto kr = [&](int a, int b, int d) {
        const T kv = c.ka[g.at(a, b, d)];
        if (b == 0) b = 1; else if (b == ny + 1) b = ny;
        if (d == 0) d = 1; else if (d == nz + 1) d = nz;
        if (a == 0) a = per ? nx : 1; else if (a == nx + 1) a = per ? 1 : nx;
        return kv * c.rho[g.at(a, b, d)];
    };
    T diff, rf, h;
    if (axis == 0) {
        diff = kr(i, j, k) - kr(i - 1, j, k);
        rf = interp_cf<T>(i, nx, per, [&](int m) { return c.rho[g.at(m, j, k)]; });
        h = T(c.dx);
    } else if (axis == 1) {
        diff = kr(i, j, k) - kr(i, j - 1, k);
        rf = interp_cf<T>(j, ny, false, [&](int m) { return c.rho[g.at(i, m, k)]; });
        h = T(c.dy);
    } else {
        diff = kr(i, j, k) - kr(i, j, k - 1);
        rf = interp_cf<T>(k, nz, false, [&](int m) { return c.rho[g.at(i, j, m)]; });
        h = T(c.dz);
    }
    return T(2. / 3.) * diff / (h * rf);
}

// SuLi-ICdz's spacing-weighted interpz_cf (SuLi-ICdz/8_derivadas.f90:450-479)
// at z face f of cells 1..n: (a(f) dz(f) + a(f-1) dz(f-1)) / (dz(f) +
// dz(f-1)) for f in 2..n, faces 1 and n+1 the copies of faces 2 and n
template <typename T, bool IN = false, typename F>
__device__ __forceinline__ T zcf_w(const CaseDev<T> &c, int f, int n, F get)
{
    const int ff = IN ? f : (f < 2 ? 2 : (f > n ? n : f));
    const double a = c.dzk[ff], b = c.dzk[ff - 1];
    return (get(ff) * T(a) + get(ff - 1) * T(b)) / T(a + b);
}
// and interpz_fc (:491-511) of a w-like array at centre kk: weights dzz
template <typename T>
__device__ __forceinline__ T zfc_w(const CaseDev<T> &c, T lo, T hi, int kk)
{
    const double a = c.dzzk[kk], b = c.dzzk[kk + 1];
    return (lo * T(a) + hi * T(b)) / T(a + b);
}

// operands gathered from the case's arrays in global memory
template <typename T>
struct GlobalAcc {
    const CaseDev<T> &c;
    __device__ __forceinline__ T u(int a, int b, int d) const { return c.u[c.g.at(a, b, d)]; }
    __device__ __forceinline__ T v(int a, int b, int d) const { return c.v[c.g.at(a, b, d)]; }
    __device__ __forceinline__ T w(int a, int b, int d) const { return c.w[c.g.at(a, b, d)]; }
    __device__ __forceinline__ T mu(int a, int b, int d) const { return c.mu[c.g.at(a, b, d)]; }
    __device__ __forceinline__ T rho(int a, int b, int d) const { return c.rho[c.g.at(a, b, d)]; }
    __device__ __forceinline__ T xmu(int a, int b, int d) const { return c.xmu[c.g.at(a, b, d)]; }
    __device__ __forceinline__ T ymu(int a, int b, int d) const { return c.ymu[c.g.at(a, b, d)]; }
    __device__ __forceinline__ T zmu(int a, int b, int d) const { return c.zmu[c.g.at(a, b, d)]; }
};

// Fu at x-face (i, j, k), i in 1..nx+1 (convdiff + classico, before complementos)
template <typename T, typename A, bool IN = false, bool VZ = false>
__device__ __forceinline__ T face_fu(const CaseDev<T> &c, const A &X, int i, int j, int k)
{
    const int nx = c.g.nx, ny = c.g.ny, nz = c.g.nz;
    // reciprocal spacings (1.0 / dx from the host); VZ: 1 / dz(k) of u's own k
    const T dx = cval<T>(c.idx, c.fidx), dy = cval<T>(c.idy, c.fidy), dz = VZ ? T(c.idzk[k]) : cval<T>(c.idz, c.fidz);
    const bool px = (c.ccx0 == 0);
    auto U = [&](int a, int b, int cc) { return X.u(a, b, cc); };
    T bma = interp_cf<T, IN>(i, nx, px, [&](int m) { return (X.v(m, j, k) + X.v(m, j + 1, k)) * T(0.5); });
    T dma = interp_cf<T, IN>(i, nx, px, [&](int m) {
        return VZ ? zfc_w<T>(c, X.w(m, j, k), X.w(m, j, k + 1), k) : (X.w(m, j, k) + X.w(m, j, k + 1)) * T(0.5);
    });
    T ddx = upw<T>(U(i, j, k), d2n<T, IN>(i, nx + 1, px, dx, [&](int m) { return U(m, j, k); }),
                   d2p<T, IN>(i, nx + 1, px, dx, [&](int m) { return U(m, j, k); }));
    T ddy = upw<T>(bma, d2n<T, IN>(j, ny, false, dy, [&](int m) { return U(i, m, k); }),
                   d2p<T, IN>(j, ny, false, dy, [&](int m) { return U(i, m, k); }));
    T ddz = upw<T>(dma, d2n<T, IN>(k, nz, false, dz, [&](int m) { return U(i, j, m); }),
                   d2p<T, IN>(k, nz, false, dz, [&](int m) { return U(i, j, m); }));
    T uint_ = ddx + ddy + ddz;
    T ama_i = X.mu(clampi_in<IN>(i, 1, nx), j, k) * dx;
    T ama_m = X.mu(clampi_in<IN>(i - 1, 1, nx), j, k) * dx;
    T b1 = interp_cf<T, IN>(j + 1, ny, false, [&](int m) { return X.xmu(i, m, k); }) * dy;
    T b0 = interp_cf<T, IN>(j, ny, false, [&](int m) { return X.xmu(i, m, k); }) * dy;
    T d1, d0;
    if (VZ) {
        // dma over dz(k) only for i <= nx, j <= ny, k <= nz; the last x face and
        // the top face keep the undivided viscosity (SuLi-ICdz/6_convdiff.f90:118-126)
        auto xm = [&](int m) { return X.xmu(i, j, m); };
        d1 = zcf_w<T, IN>(c, k + 1, nz, xm) * ((i <= nx && k + 1 <= nz) ? T(c.idzk[k + 1]) : T(1.));
        d0 = zcf_w<T, IN>(c, k, nz, xm) * ((i <= nx) ? T(c.idzk[k]) : T(1.));
    } else {
        d1 = interp_cf<T, IN>(k + 1, nz, false, [&](int m) { return X.xmu(i, j, m); }) * dz;
        d0 = interp_cf<T, IN>(k, nz, false, [&](int m) { return X.xmu(i, j, m); }) * dz;
    }
    T rhox = interp_cf<T, IN>(i, nx, px, [&](int m) { return X.rho(m, j, k); });
    T uc = U(i, j, k);
    const T rrho = T(1.) / rhox;
    return -uint_ +
           ((ama_i * T(2.) * (U(i + 1, j, k) - uc) - ama_m * T(2.) * (uc - U(i - 1, j, k))) * dx +
            b1 * ((U(i, j + 1, k) - uc) * dy + (X.v(i, j + 1, k) - X.v(i - 1, j + 1, k)) * dx) -
            b0 * ((uc - U(i, j - 1, k)) * dy + (X.v(i, j, k) - X.v(i - 1, j, k)) * dx) +
            d1 * ((U(i, j, k + 1) - uc) * dz + (X.w(i, j, k + 1) - X.w(i - 1, j, k + 1)) * dx) -
            d0 * ((uc - U(i, j, k - 1)) * dz + (X.w(i, j, k) - X.w(i - 1, j, k)) * dx)) *
               rrho;
}

// Fv at y-face (i, j, k), j in 1..ny+1
template <typename T, typename A, bool IN = false, bool VZ = false>
__device__ __forceinline__ T face_fv(const CaseDev<T> &c, const A &X, int i, int j, int k)
{
    const int nx = c.g.nx, ny = c.g.ny, nz = c.g.nz;
    const T dx = cval<T>(c.idx, c.fidx), dy = cval<T>(c.idy, c.fidy), dz = VZ ? T(c.idzk[k]) : cval<T>(c.idz, c.fidz);
    const bool px = (c.ccx0 == 0);
    auto V = [&](int a, int b, int cc) { return X.v(a, b, cc); };
    T amb = interp_cf<T, IN>(j, ny, false, [&](int m) { return (X.u(i, m, k) + X.u(i + 1, m, k)) * T(0.5); });
    T dmb = interp_cf<T, IN>(j, ny, false, [&](int m) {
        return VZ ? zfc_w<T>(c, X.w(i, m, k), X.w(i, m, k + 1), k) : (X.w(i, m, k) + X.w(i, m, k + 1)) * T(0.5);
    });
    T ddx = upw<T>(amb, d2n<T, IN>(i, nx, px, dx, [&](int m) { return V(m, j, k); }),
                   d2p<T, IN>(i, nx, px, dx, [&](int m) { return V(m, j, k); }));
    T ddy = upw<T>(V(i, j, k), d2n<T, IN>(j, ny + 1, false, dy, [&](int m) { return V(i, m, k); }),
                   d2p<T, IN>(j, ny + 1, false, dy, [&](int m) { return V(i, m, k); }));
    T ddz = upw<T>(dmb, d2n<T, IN>(k, nz, false, dz, [&](int m) { return V(i, j, m); }),
                   d2p<T, IN>(k, nz, false, dz, [&](int m) { return V(i, j, m); }));
    T vint = ddx + ddy + ddz;
    T a1 = interp_cf<T, IN>(i + 1, nx, px, [&](int m) { return X.ymu(m, j, k); }) * dx;
    T a0 = interp_cf<T, IN>(i, nx, px, [&](int m) { return X.ymu(m, j, k); }) * dx;
    T bmb_j = X.mu(i, clampi_in<IN>(j, 1, ny), k) * dy;
    T bmb_m = X.mu(i, clampi_in<IN>(j - 1, 1, ny), k) * dy;
    T d1, d0;
    if (VZ) {
        // dmb over dz(k) only for j <= ny, k <= nz (SuLi-ICdz/6_convdiff.f90:118-126)
        auto ym = [&](int m) { return X.ymu(i, j, m); };
        d1 = zcf_w<T, IN>(c, k + 1, nz, ym) * ((j <= ny && k + 1 <= nz) ? T(c.idzk[k + 1]) : T(1.));
        d0 = zcf_w<T, IN>(c, k, nz, ym) * ((j <= ny) ? T(c.idzk[k]) : T(1.));
    } else {
        d1 = interp_cf<T, IN>(k + 1, nz, false, [&](int m) { return X.ymu(i, j, m); }) * dz;
        d0 = interp_cf<T, IN>(k, nz, false, [&](int m) { return X.ymu(i, j, m); }) * dz;
    }
    T rhoy = interp_cf<T, IN>(j, ny, false, [&](int m) { return X.rho(i, m, k); });
    T vc = V(i, j, k);
    return -vint +
           (a1 * ((V(i + 1, j, k) - vc) * dx + (X.u(i + 1, j, k) - X.u(i + 1, j - 1, k)) * dy) -
            a0 * ((vc - V(i - 1, j, k)) * dx + (X.u(i, j, k) - X.u(i, j - 1, k)) * dy) +
            (bmb_j * T(2.) * (V(i, j + 1, k) - vc) - bmb_m * T(2.) * (vc - V(i, j - 1, k))) * dy +
            d1 * ((V(i, j, k + 1) - vc) * dz + (X.w(i, j, k + 1) - X.w(i, j - 1, k + 1)) * dy) -
            d0 * ((vc - V(i, j, k - 1)) * dz + (X.w(i, j, k) - X.w(i, j - 1, k)) * dy)) /
               rhoy;
}

// Fw at z-face (i, j, k), k in 1..nz+1
template <typename T, typename A, bool IN = false, bool VZ = false>
__device__ __forceinline__ T face_fw(const CaseDev<T> &c, const A &X, int i, int j, int k)
{
    const int nx = c.g.nx, ny = c.g.ny, nz = c.g.nz;
    // VZ: the z differences of u, v over dz(k), those of w over dzz(k)
    const T dx = cval<T>(c.idx, c.fidx), dy = cval<T>(c.idy, c.fidy), dz = VZ ? T(c.idzk[k]) : cval<T>(c.idz, c.fidz);
    const T dzw = VZ ? T(c.idzzk[k]) : dz;
    const bool px = (c.ccx0 == 0);
    auto W = [&](int a, int b, int cc) { return X.w(a, b, cc); };
    auto ua = [&](int m) { return (X.u(i, j, m) + X.u(i + 1, j, m)) * T(0.5); };
    auto va = [&](int m) { return (X.v(i, j, m) + X.v(i, j + 1, m)) * T(0.5); };
    T amd = VZ ? zcf_w<T, IN>(c, k, nz, ua) : interp_cf<T, IN>(k, nz, false, ua);
    T bmd = VZ ? zcf_w<T, IN>(c, k, nz, va) : interp_cf<T, IN>(k, nz, false, va);
    T ddx = upw<T>(amd, d2n<T, IN>(i, nx, px, dx, [&](int m) { return W(m, j, k); }),
                   d2p<T, IN>(i, nx, px, dx, [&](int m) { return W(m, j, k); }));
    T ddy = upw<T>(bmd, d2n<T, IN>(j, ny, false, dy, [&](int m) { return W(i, m, k); }),
                   d2p<T, IN>(j, ny, false, dy, [&](int m) { return W(i, m, k); }));
    T ddz = upw<T>(W(i, j, k), d2n<T, IN>(k, nz + 1, false, dzw, [&](int m) { return W(i, j, m); }),
                   d2p<T, IN>(k, nz + 1, false, dzw, [&](int m) { return W(i, j, m); }));
    T wint = ddx + ddy + ddz;
    T a1 = interp_cf<T, IN>(i + 1, nx, px, [&](int m) { return X.zmu(m, j, k); }) * dx;
    T a0 = interp_cf<T, IN>(i, nx, px, [&](int m) { return X.zmu(m, j, k); }) * dx;
    T b1 = interp_cf<T, IN>(j + 1, ny, false, [&](int m) { return X.zmu(i, m, k); }) * dy;
    T b0 = interp_cf<T, IN>(j, ny, false, [&](int m) { return X.zmu(i, m, k); }) * dy;
    const int kc = clampi_in<IN>(k, 1, nz), km = clampi_in<IN>(k - 1, 1, nz);
    // VZ: dmd = mu / dzz(k) (SuLi-ICdz/6_convdiff.f90:120)
    T dmd_k = X.mu(i, j, kc) * (VZ ? T(c.idzzk[kc]) : dz);
    T dmd_m = X.mu(i, j, km) * (VZ ? T(c.idzzk[km]) : dz);
    auto rr = [&](int m) { return X.rho(i, j, m); };
    T rhoz = VZ ? zcf_w<T, IN>(c, k, nz, rr) : interp_cf<T, IN>(k, nz, false, rr);
    T wc = W(i, j, k);
    return -wint +
           (a1 * ((W(i + 1, j, k) - wc) * dx + (X.u(i + 1, j, k) - X.u(i + 1, j, k - 1)) * dz) -
            a0 * ((wc - W(i - 1, j, k)) * dx + (X.u(i, j, k) - X.u(i, j, k - 1)) * dz) +
            b1 * ((W(i, j + 1, k) - wc) * dy + (X.v(i, j + 1, k) - X.v(i, j + 1, k - 1)) * dz) -
            b0 * ((wc - W(i, j - 1, k)) * dy + (X.v(i, j, k) - X.v(i, j, k - 1)) * dz) +
            (dmd_k * T(2.) * (W(i, j, k + 1) - wc) - dmd_m * T(2.) * (wc - W(i, j, k - 1))) * dzw) /
               rhoz;
}

// the complementos terms fused after each face's convdiff value, in the
// reference's order: gravity (x, z), the sponge (w), surface tension, the
// manufactured source (only where mms_t != 0: elsewhere tf_* is zero), the
// kinetic-energy term
template <typename T>
__device__ __forceinline__ T compl_fu(const CaseDev<T> &c, T F, int i, int j, int k)
{
    const Geo &g = c.g;
    F = F + T(c.gx);
    if (c.t_tens == 1) F = F - tension_face(c, 0, i, j, k);
    if (c.mms_t != 0) F = F + c.tf_u[g.at(i, j, k)];
    if (c.m_turb >= 2) F = F - ka_face(c, 0, i, j, k);
    return F;
}
template <typename T>
__device__ __forceinline__ T compl_fv(const CaseDev<T> &c, T F, int i, int j, int k)
{
    const Geo &g = c.g;
    if (c.t_tens == 1) F = F - tension_face(c, 1, i, j, k);
    if (c.mms_t != 0) F = F + c.tf_v[g.at(i, j, k)];
    if (c.m_turb >= 2) F = F - ka_face(c, 1, i, j, k);
    return F;
}
template <typename T>
__device__ __forceinline__ T compl_fw(const CaseDev<T> &c, T F, T wc, int i, int j, int k)
{
    const Geo &g = c.g;
    F = F - T(c.gz);
    if (c.epis) F = F - (wc - T(0.)) * c.epis[g.at(i, j, k)];
    if (c.t_tens == 1) F = F - tension_face(c, 2, i, j, k);
    if (c.mms_t != 0) F = F + c.tf_w[g.at(i, j, k)];
    if (c.m_turb >= 2) F = F - ka_face(c, 2, i, j, k);
    return F;
}

}  // namespace suli
