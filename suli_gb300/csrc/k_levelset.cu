// k_levelset.cu -- level-set kernels: WENO5 advection (TVD-RK3), the
// reinitialisation loop, Heaviside / properties and the FP64 volume integral.
//
// Replaces 14_level_set.f90:204-594 and 8_derivadas.f90:675-1095.  The WENO
// halos (3 cells, built by extrapolation or the node-style periodic wrap in
// wenox/y/z) are formed on the fly from the 7-point line each thread loads,
// so no halo array or fill pass is needed.  The three RK stages rotate
// through ls -> lsb -> lsc -> ls, so stage 3 writes the result back in place
// (each thread reads ls only at its own cell in stages 2/3) and ls0 = ls is
// never copied.
#include "suli_kernels.cuh"

namespace suli {

// Jiang-Shu WENO5 on five one-sided differences (8_derivadas.f90:778-806)
template <typename T>
__device__ __forceinline__ T weno5(T v0, T v1, T v2, T v3, T v4)
{
    // Jiang-Shu WENO5 (8_derivadas.f90:778-806).  The nonlinear weights
    // om_k = (c_k/q_k) / sum_j (c_j/q_j), q_k = (eps + IS_k)^2, are formed as
    // c_k P_k / sum_j c_j P_j with P_k the product of the other two q's:
    // algebraically the reference's weights, one division instead of six.
    const T aux1 = T(13. / 12.), aux2 = T(1. / 4.), aux3 = T(1. / 6.), aux6 = T(0.00000001);
    T a, b;
    a = v0 - 2 * v1 + v2;
    b = v0 - 4 * v1 + 3 * v2;
    T is1 = aux1 * a * a + aux2 * b * b;
    a = v1 - 2 * v2 + v3;
    b = v1 - v3;
    T is2 = aux1 * a * a + aux2 * b * b;
    a = v2 - 2 * v3 + v4;
    b = 3 * v2 - 4 * v3 + v4;
    T is3 = aux1 * a * a + aux2 * b * b;
    T q1 = (aux6 + is1) * (aux6 + is1);
    T q2 = (aux6 + is2) * (aux6 + is2);
    T q3 = (aux6 + is3) * (aux6 + is3);
    T w1 = T(0.1) * (q2 * q3), w2 = T(0.6) * (q1 * q3), w3 = T(0.3) * (q1 * q2);
    // the correctly rounded reciprocal (the value of 1 / x)
    T inv;
    if constexpr (sizeof(T) == 4) inv = __frcp_rn(w1 + w2 + w3);
    else inv = T(1.) / (w1 + w2 + w3);
    return aux3 * inv * (w1 * (2 * v0 - 7 * v1 + 11 * v2) + w2 * (-v1 + 5 * v2 + 2 * v3) +
                         w3 * (2 * v2 + 5 * v3 - v4));
}

// Load phi(m), m = i-3..i+3, of one grid line (element m at base + m*st),
// (ihs = 1, the curvature's mode, extrapolates the low end differently),
// building the out-of-range values as wenox/y/z do: ihs = 0 periodic with
// phi(0) = phi(n-1) etc. (:702-714), otherwise cubic extrapolation (:742-756).
template <typename T>
__device__ __forceinline__ void load_line(const T *__restrict__ a, long long base, long long st, int i, int n,
                                          int ihs, T (&L)[7])
{
    // one 64-bit base, then 32-bit offsets: a case box holds fewer than 2^31
    // elements (suli_create refuses larger ones)
    const T *__restrict__ p = a + base;
    const int s = (int)st;
    if (i >= 4 && i <= n - 3) {
        const T *__restrict__ q = p + (i - 3) * s;
#pragma unroll
        for (int t = 0; t < 7; ++t) L[t] = q[t * s];
        return;
    }
#pragma unroll
    for (int t = 0; t < 7; ++t) {
        int m = i - 3 + t;
        if (ihs == 0) {
            if (m < 1) m += n - 1;
            else if (m > n) m -= n - 1;
            L[t] = p[m * s];
        } else if (m >= 1 && m <= n) {
            L[t] = p[m * s];
        }
    }
    if (ihs != 0) {
        const T c11 = T(1. / 11.);
        if (i - 3 < 1) {
            // ihs = 1 (curv_ls1): the low end's weights are (12, -9, 2) / 5
            // (8_derivadas.f90:716-721); ihs = 2: (18, -9, 2) / 11
            const T cl = (ihs == 1) ? T(1. / 5.) : c11, w0 = (ihs == 1) ? T(12.) : T(18.);
            T p1 = p[s], p2 = p[2 * s], p3 = p[3 * s];
            T g0 = cl * (w0 * p1 - T(9.) * p2 + T(2.) * p3);
            T gm1 = cl * (w0 * g0 - T(9.) * p1 + T(2.) * p2);
            T gm2 = cl * (w0 * gm1 - T(9.) * g0 + T(2.) * p1);
#pragma unroll
            for (int t = 0; t < 7; ++t) {
                int m = i - 3 + t;
                if (m == 0) L[t] = g0;
                else if (m == -1) L[t] = gm1;
                else if (m == -2) L[t] = gm2;
            }
        }
        if (i + 3 > n) {
            T pn = p[n * s], pn1 = p[(n - 1) * s], pn2 = p[(n - 2) * s];
            T g1 = c11 * (T(18.) * pn - T(9.) * pn1 + T(2.) * pn2);
            T g2 = c11 * (T(18.) * g1 - T(9.) * pn + T(2.) * pn1);
            T g3 = c11 * (T(18.) * g2 - T(9.) * g1 + T(2.) * pn);
#pragma unroll
            for (int t = 0; t < 7; ++t) {
                int m = i - 3 + t;
                if (m == n + 1) L[t] = g1;
                else if (m == n + 2) L[t] = g2;
                else if (m == n + 3) L[t] = g3;
            }
        }
    }
}

// rh = 1/h (the host's 1.0 / h, rounded to T)
template <typename T>
__device__ __forceinline__ void weno_pm(const T (&L)[7], T rh, T &dp, T &dn)
{
    T D[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) D[t] = (L[t + 1] - L[t]) * rh;
    dp = weno5<T>(D[5], D[4], D[3], D[2], D[1]);
    dn = weno5<T>(D[0], D[1], D[2], D[3], D[4]);
}

// der_weno (14_level_set.f90:338-370) at cell (i,j,k) of a cell array with
// interior dims (n0,n1,n2): returns x+, x-, y+, y-, z+, z-.
template <typename T>
__device__ __forceinline__ void der_weno_at(const CaseDev<T> &c, const T *__restrict__ a, int i, int j, int k,
                                            int n0, int n1, int n2, T &xp, T &xm, T &yp, T &ym, T &zp, T &zm)
{
    const Geo &g = c.g;
    T L[7];
    load_line<T>(a, g.at(0, j, k), 1, i, n0, c.ccx0 == 0 ? 0 : 2, L);
    weno_pm<T>(L, cval<T>(c.idx, c.fidx), xp, xm);
    load_line<T>(a, g.at(i, 0, k), g.sx, j, n1, c.ccy0 == 0 ? 0 : 2, L);
    weno_pm<T>(L, cval<T>(c.idy, c.fidy), yp, ym);
    load_line<T>(a, g.at(i, j, 0), g.sxy, k, n2, 2, L);
    if (c.dz11 != nullptr) {
        // SuLi-ICdz's wenoz: the differences over the extrapolated spacing,
        // D = (phi(m+1) - phi(m)) / dz11(m+1), m = k-3 .. k+2
        // (SuLi-ICdz/8_derivadas.f90:1090-1102)
        T D[6];
#pragma unroll
        for (int t = 0; t < 6; ++t) D[t] = (L[t + 1] - L[t]) / T(c.dz11[k - 2 + t]);
        zp = weno5<T>(D[5], D[4], D[3], D[2], D[1]);
        zm = weno5<T>(D[0], D[1], D[2], D[3], D[4]);
        return;
    }
    weno_pm<T>(L, cval<T>(c.idz, c.fidz), zp, zm);
}
template <typename T>
__device__ __forceinline__ void der_weno_at(const CaseDev<T> &c, const T *__restrict__ a, int i, int j, int k,
                                            T &xp, T &xm, T &yp, T &ym, T &zp, T &zm)
{
    der_weno_at<T>(c, a, i, j, k, c.g.nx, c.g.ny, c.g.nz, xp, xm, yp, ym, zp, zm);
}

// level-set array the reinitialisation acts on: 0 = ls, 1..4 = the obstacle
// level sets obs_lsx/obs_lsy/obs_lsz/obs_lss (obstaculo(), 3_contorno.f90:991-996)
template <typename T>
__device__ __forceinline__ T *reinit_target(const CaseDev<T> &c, int target, int &n0, int &n1, int &n2)
{
    n0 = c.g.nx; n1 = c.g.ny; n2 = c.g.nz;
    switch (target) {
    case 1: n0 += 1; return c.obs_lsx;
    case 2: n1 += 1; return c.obs_lsy;
    case 3: n2 += 1; return c.obs_lsz;
    case 4: return c.obs_lss;
    default: return c.ls;
    }
}

// Godunov |grad phi| of reinic_weno (:397-421)
template <typename T>
__device__ __forceinline__ T godunov(T ls, T ta, T tb, T tc, T td, T te, T tf)
{
    const T eps = T(0.00000001);
    T a1, a2, A, B, C;
    if (ls > T(0.)) {
        a1 = fmax(td, eps); a2 = -fmin(ta, eps); A = fmax(a1, a2);
        a1 = fmax(te, eps); a2 = -fmin(tb, eps); B = fmax(a1, a2);
        a1 = fmax(tf, eps); a2 = -fmin(tc, eps); C = fmax(a1, a2);
    } else {
        a1 = fmax(ta, eps); a2 = -fmin(td, eps); A = fmax(a1, a2);
        a1 = fmax(tb, eps); a2 = -fmin(te, eps); B = fmax(a1, a2);
        a1 = fmax(tc, eps); a2 = -fmin(tf, eps); C = fmax(a1, a2);
    }
    return sqrt(A * A + B * B + C * C);
}

template <typename T>
__device__ __forceinline__ void stage_bufs(const CaseDev<T> &c, T *base, int stage, const T *&src, T *&dst)
{
    if (stage == 1) { src = base; dst = c.lsb; }
    else if (stage == 2) { src = c.lsb; dst = c.lsc; }
    else { src = c.lsc; dst = base; }
}

// the FP64 masters of the same rotation (mixed form, target 0)
template <typename T>
__device__ __forceinline__ void stage_bufs64(const CaseDev<T> &c, int stage, const double *&src, double *&dst)
{
    if (stage == 1) { src = c.ls64; dst = c.lsb64; }
    else if (stage == 2) { src = c.lsb64; dst = c.lsc64; }
    else { src = c.lsc64; dst = c.ls64; }
}

// conv_weno + intt_ls (14_level_set.f90:277-334), one TVD-RK3 stage
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_ls_adv_stage(const CaseDev<T> *__restrict__ cs, int ncases, int stage,
                                                           const double *__restrict__ rk)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const T *src;
    T *dst;
    stage_bufs(c, c.ls, stage, src, dst);
    long long q = g.at(i, j, k);
    T ta, td, tb, te, tc, tf;
    der_weno_at<T>(c, src, i, j, k, ta, td, tb, te, tc, tf);
    T ua = (c.u[q] + c.u[q + 1]) * T(0.5);
    T va = (c.v[q] + c.v[q + g.sx]) * T(0.5);
    T wa = (c.w[q] + c.w[q + g.sxy]) * T(0.5);
    T apos = ua > T(0.) ? ua : T(0.), aneg = ua < T(0.) ? ua : T(0.);
    T bpos = va > T(0.) ? va : T(0.), bneg = va < T(0.) ? va : T(0.);
    T cpos = wa > T(0.) ? wa : T(0.), cneg = wa < T(0.) ? wa : T(0.);
    T sy7 = -(apos * td + aneg * ta + bpos * te + bneg * tb + cpos * tf + cneg * tc);
    if (c.ls64 != nullptr) {   // mixed form: the stage combination on the FP64 masters
        const double *s64;
        double *d64;
        stage_bufs64(c, stage, s64, d64);
        const double nv = rk[stage - 1] * c.ls64[q] + rk[3 + stage - 1] * s64[q] +
                          rk[6 + stage - 1] * c.sc[S_DTADV] * (double)sy7;
        d64[q] = nv;
        dst[q] = T(nv);
        return;
    }
    T ta1 = c.ls[q];          // ls0 (stage 1: the current value)
    T gx = src[q];
    T dt1 = T(c.sc[S_DTADV]);
    T a = T(rk[stage - 1]), b = T(rk[3 + stage - 1]), gg = T(rk[6 + stage - 1]);
    dst[q] = a * ta1 + b * gx + gg * dt1 * sy7;
}

// func_s of reinic_weno (:391-426); also resets the loop state of the case
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_reinit_funcs(const CaseDev<T> *__restrict__ cs, int ncases, int target)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (blockIdx.x == c.tile_begin && tid_lin() == 0) {
        c.sc[S_RINACTIVE] = (target == 0 || c.ibm_t == 2) ? 1.0 : 0.0;
        c.sc[S_RINITER] = 0.0;
    }
    int n0, n1, n2;
    const T *a = reinit_target(c, target, n0, n1, n2);
    if (i > n0 || j > n1 || k > n2) return;
    if (target != 0 && c.ibm_t != 2) return;
    long long q = g.at(i, j, k);
    T ta, td, tb, te, tc, tf;
    der_weno_at<T>(c, a, i, j, k, n0, n1, n2, ta, td, tb, te, tc, tf);
    T lv = a[q];
    T mod = godunov<T>(lv, ta, tb, tc, td, te, tf);
    T dx1 = T(c.dx1);
    c.funcs[q] = lv / sqrt(lv * lv + mod * mod * dx1 * dx1);
}

// one RK stage of the reinitialisation iteration `iter` (:431-500); stage 3
// also forms the signed band error and decides whether to iterate again.
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_reinit_stage(const CaseDev<T> *__restrict__ cs, int ncases, int stage,
                                                           int iter, const double *__restrict__ rk, int target)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_RINACTIVE] == 0.0) return;      // loop of this case has ended
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    int n0, n1, n2;
    T *base = reinit_target(c, target, n0, n1, n2);
    bool in = (i <= n0 && j <= n1 && k <= n2);
    const T *src;
    T *dst;
    stage_bufs(c, base, stage, src, dst);
    T band = T(0), cnt = T(0);     // stage 3: the band's change and cell count
    if (in) {
        long long q = g.at(i, j, k);
        T ta, td, tb, te, tc, tf;
        der_weno_at<T>(c, src, i, j, k, n0, n1, n2, ta, td, tb, te, tc, tf);
        T lv = src[q];
        T mod = godunov<T>(lv, ta, tb, tc, td, te, tf);
        T sy7 = c.funcs[q] * (T(1.) - mod);
        double nv64, lv64;
        if (target == 0 && c.ls64 != nullptr) {
            // mixed form: the stage combination on the FP64 masters
            const double *s64;
            double *d64;
            stage_bufs64(c, stage, s64, d64);
            lv64 = s64[q];
            nv64 = rk[stage - 1] * c.ls64[q] + rk[3 + stage - 1] * lv64 + rk[6 + stage - 1] * c.dt1 * (double)sy7;
            d64[q] = nv64;
            dst[q] = T(nv64);
        } else {
            T ta1 = base[q];
            T a = T(rk[stage - 1]), b = T(rk[3 + stage - 1]), gg = T(rk[6 + stage - 1]);
            T nv = a * ta1 + b * lv + gg * T(c.dt1) * sy7;
            dst[q] = nv;
            nv64 = (double)nv;
            lv64 = (double)lv;
        }
        if (stage == 3) {
            if (fabs(nv64) <= 2. * c.alpha1 * c.dx1) {
                band = T(nv64 - lv64);
                cnt = T(1);
            }
        }
    }
    if (stage != 3) return;
    double tot[2];
    bool last;
    if constexpr (sizeof(T) == 4) {
        // mixed form: FP32 warp sums of the band's changes (the stopping
        // test's mean change) and counts (exact)
        const float vals[2] = {band, cnt};
        const double one[2] = {1.0, 1.0};
        last = last_block_reduce_f32<T, 2>(c, vals, one, tot);
    } else {
        const double vals[2] = {band, cnt};
        last = last_block_reduce<T, 2>(c, vals, tot);
    }
    if (last && tid_lin() == 0) {
        double il = (double)iter;
        double active;
        double replay = c.sc[S_RINREPLAY];
        if (replay >= 0.0) active = (il < replay) ? 1.0 : 0.0;
        else if (iter == c.reinit_max) active = 0.0;
        else {
            double err = tot[0] / tot[1];
            active = (err > c.dt1 * c.dx1 * c.dx1) ? 1.0 : 0.0;
        }
        c.sc[S_RINITER] = il;
        c.sc[S_RINACTIVE] = active;
    }
}

// heaviside (14_level_set.f90:508-594, t_tens = 0) + the volume sum
// (:233-240); the last block decides whether the volume correction runs.
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_heaviside_vol(const CaseDev<T> *__restrict__ cs, int ncases, int set_ini)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    double vol = 0.0;
    float hf = 0.f;     // mixed form: the cell's H for an FP32 warp sum
    if (i <= g.nx && j <= g.ny && k <= g.nz) {
        long long q = g.at(i, j, k);
        T l = c.ls[q];
        const double lm = c.ls64 ? c.ls64[q] : (double)l;   // FP64 master in the mixed form
        T ad = T(c.alpha1 * c.dx1);
        T h;
        if (l < -ad) h = T(0.);
        else if (l > ad) h = T(1.);
        else h = T(0.5) * (T(1.) + l / ad + T(1. / c.pi) * sin(T(c.pi) * l / ad));
        c.hs[q] = h;
        c.rho[q] = T(c.rho_f1) * (T(1.) - h) + T(c.rho_f2) * h;
        double hv = (double)h;
        if (c.rho64) {
            // mixed form: Heaviside of the FP64 level-set master in FP64, for
            // the density of the FP64 pressure operator and the volume integral
            // (l / ad by the reciprocal: no FP64 divide, a long sequence on
            // GB300's FP64 units)
            double l64 = lm, ad64 = c.alpha1 * c.dx1, h64;
            if (l64 < -ad64) h64 = 0.;
            else if (l64 > ad64) h64 = 1.;
            else {
                const double la = l64 * rcp_nr64(ad64);
                h64 = 0.5 * (1. + la + 1. / c.pi * sin(c.pi * la));
            }
            c.rho64[q] = c.rho_f1 * (1. - h64) + c.rho_f2 * h64;
            hv = h64;
        }
        c.ls_mu[q] = T(c.mu_f1) * (T(1.) - h) + T(c.mu_f2) * h;
        if (c.t_tens == 1) {
            // surface-tension weights (14_level_set.f90:519-546, :563-567):
            // the larger one-sided WENO derivative of ls times the smoothed
            // delta, zero outside the band
            T ta, td, tb, te, tc, tf;
            der_weno_at<T>(c, c.ls, i, j, k, ta, td, tb, te, tc, tf);
            const T ga = (fabs(ta) > fabs(td)) ? ta : td;
            const T gb = (fabs(tb) > fabs(te)) ? tb : te;
            const T gc = (fabs(tc) > fabs(tf)) ? tc : tf;
            T sx = T(0.), sy = T(0.), sz = T(0.);
            if (!(l < -ad) && !(l > ad)) {
                sx = T(0.5) * ga * (T(1.) + cos(T(c.pi) * l / ad)) / ad;
                sy = T(0.5) * gb * (T(1.) + cos(T(c.pi) * l / ad)) / ad;
                sz = T(0.5) * gc * (T(1.) + cos(T(c.pi) * l / ad)) / ad;
            }
            c.hsx[q] = sx;
            c.hsy[q] = sy;
            c.hsz[q] = sz;
        }
        if constexpr (sizeof(T) == 4) hf = (float)hv;
        else vol = (1. - (1. - hv)) * c.dx * c.dy * (c.dzk ? c.dzk[k] : c.dz);   // SuLi-ICdz/14_level_set.f90:176,222
    }
    if (set_ini < 0) return;     // properties only (heaviside after the level-set IBM)
    double tot[1];
    bool last;
    if constexpr (sizeof(T) == 4) {
        // mixed form: H summed in FP32 along each warp (an x-row of the tile:
        // one cell volume), times the cell volume once per warp
        const float vals[1] = {hf};
        const double cv[1] = {c.dx * c.dy * (c.dzk ? c.dzk[min(k, g.nz)] : c.dz)};
        last = last_block_reduce_f32<T, 1>(c, vals, cv, tot);
    } else {
        const double vals[1] = {vol};
        last = last_block_reduce<T, 1>(c, vals, tot);
    }
    if (last && tid_lin() == 0) {
        double vi = tot[0];
        if (set_ini) c.sc[S_VOLINI] = vi;
        c.sc[S_VOLINS] = vi;
        double v0 = c.sc[S_VOLINI];
        c.sc[S_VOLACTIVE] = (fabs(vi - v0) / vi > 0.1 && c.mms_t != 2) ? 1.0 : 0.0;
    }
}

// volume correction update (:245-255): ls - dt1*(vol_ins-vol_ini)*|grad ls|/vol_ini
// with |grad ls| from mod_ls1 (:598-655); writes lsb, copied back after.
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_volcorr(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_VOLACTIVE] == 0.0) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    long long q = g.at(i, j, k);
    T ta, td, tb, te, tc, tf;
    der_weno_at<T>(c, c.ls, i, j, k, ta, td, tb, te, tc, tf);
    if (!(fabs(ta) > fabs(td))) ta = td;
    if (!(fabs(tb) > fabs(te))) tb = te;
    if (!(fabs(tc) > fabs(tf))) tc = tf;
    T m = sqrt(ta * ta + tb * tb + tc * tc);
    double vi = c.sc[S_VOLINS], v0 = c.sc[S_VOLINI];
    if (c.ls64 != nullptr) {
        const double x = c.ls64[q] - c.dt1 * (vi - v0) * (double)m / v0;
        c.lsb64[q] = x;
        c.lsb[q] = T(x);
        return;
    }
    c.lsb[q] = c.ls[q] - T(c.dt1) * T(vi - v0) * m / T(v0);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_volcorr_copy(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_VOLACTIVE] == 0.0) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    long long q = g.at(i, j, k);
    c.ls[q] = c.lsb[q];
    if (c.ls64 != nullptr) c.ls64[q] = c.lsb64[q];
}

// ---- surface tension (t_tens = 1) -------------------------------------------
// mod_ls1 (14_level_set.f90:598-655) on ls: the unit normal from the larger
// one-sided WENO derivatives (zero where the gradient vanishes)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_ls_normals(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.t_tens != 1) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    T ta, td, tb, te, tc, tf;
    der_weno_at<T>(c, c.ls, i, j, k, ta, td, tb, te, tc, tf);
    const T a = (fabs(ta) > fabs(td)) ? ta : td;
    const T b = (fabs(tb) > fabs(te)) ? tb : te;
    const T cc = (fabs(tc) > fabs(tf)) ? tc : tf;
    const T m = sqrt(a * a + b * b + cc * cc);
    const long long q = g.at(i, j, k);
    if (m == T(0)) {
        c.nlx[q] = T(0.); c.nly[q] = T(0.); c.nlz[q] = T(0.);
    } else {
        c.nlx[q] = a / m; c.nly[q] = b / m; c.nlz[q] = cc / m;
    }
}

// curv_ls1 (14_level_set.f90:660-704): each normal component differentiated
// along its own axis by WENO with the low end extrapolated as ihs = 1, the
// larger one-sided derivative of each (ties to the + side), summed
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_ls_curv(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.t_tens != 1) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    T L[7], p, n;
    load_line<T>(c.nlx, g.at(0, j, k), 1, i, g.nx, 1, L);
    weno_pm<T>(L, cval<T>(c.idx, c.fidx), p, n);
    const T ddx = (fabs(n) > fabs(p)) ? n : p;
    load_line<T>(c.nly, g.at(i, 0, k), g.sx, j, g.ny, 1, L);
    weno_pm<T>(L, cval<T>(c.idy, c.fidy), p, n);
    const T ddy = (fabs(n) > fabs(p)) ? n : p;
    load_line<T>(c.nlz, g.at(i, j, 0), g.sxy, k, g.nz, 1, L);
    weno_pm<T>(L, cval<T>(c.idz, c.fidz), p, n);
    const T ddz = (fabs(n) > fabs(p)) ? n : p;
    c.kurv[g.at(i, j, k)] = ddx + ddy + ddz;
}

// ---- host launchers -------------------------------------------------------
template <typename T>
void launch_curvature(const Batch<T> &b, cudaStream_t s)
{
    k_ls_normals<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_ls_curv<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}

template <typename T>
void launch_level_set_adv(const Batch<T> &b, cudaStream_t s)
{
    for (int st = 1; st <= 3; ++st)
        k_ls_adv_stage<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, st, b.drk); count_launch();
}

template <typename T>
void launch_reinit(const Batch<T> &b, int max_iter, cudaStream_t s, int target)
{
    k_reinit_funcs<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, target); count_launch();
    for (int it = 1; it <= max_iter; ++it)
        for (int st = 1; st <= 3; ++st) {
            k_reinit_stage<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, st, it, b.drk, target);
            count_launch();
        }
}

template <typename T>
void launch_heaviside(const Batch<T> &b, int set_ini, cudaStream_t s)
{
    k_heaviside_vol<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, set_ini); count_launch();
}

template <typename T>
void launch_volcorr(const Batch<T> &b, cudaStream_t s)
{
    k_volcorr<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_volcorr_copy<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_heaviside_vol<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 0); count_launch();
}

template void launch_level_set_adv<double>(const Batch<double> &, cudaStream_t);
template void launch_reinit<double>(const Batch<double> &, int, cudaStream_t, int);
template void launch_heaviside<double>(const Batch<double> &, int, cudaStream_t);
template void launch_volcorr<double>(const Batch<double> &, cudaStream_t);
template void launch_level_set_adv<float>(const Batch<float> &, cudaStream_t);
template void launch_reinit<float>(const Batch<float> &, int, cudaStream_t, int);
template void launch_heaviside<float>(const Batch<float> &, int, cudaStream_t);
template void launch_volcorr<float>(const Batch<float> &, cudaStream_t);
template void launch_curvature<double>(const Batch<double> &, cudaStream_t);
template void launch_curvature<float>(const Batch<float> &, cudaStream_t);

}  // namespace suli
