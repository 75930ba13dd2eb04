// k_cg.cu -- graddin() (9_grad.f90:10-663): Jacobi-scaled conjugate
// gradients for the pressure Poisson equation, and the FP64 iterative
// refinement around an FP32 inner CG used by the mixed form.
//
// Setup (once per solve):
//   k_cg_setup1  face coefficients s = dt/(h^2 rho_face) (:95-148), diagonal
//                D = sum of the six (:153-160), rhs q = -div u* (:163-183)
//   k_cg_setup2  symmetric scaling s/sqrt(D_i D_j) (:256-287), e = prd1 sqrt(D)
//                (:245-251), b = q/sqrt(D)
//   k_cg_setup3  r0 = A e - b (:292-300), p = r0, r0.r0 and the stop threshold
// Iteration (the loop of :398-587):
//   k_cg_A       mp = A p and p.mp; the case's last block forms alpha
//   k_cg_B       e -= alpha p, r -= alpha mp and r.r; last block forms beta,
//                counts the iteration and clears the case's active flag on
//                convergence (so finished cases drop out of later launches)
//   k_cg_C       p = r + beta p
// Finish: prd1 = e / sqrt(D) (:650-659) on the interior and on every ghost,
// each ghost taking the value of the interior cell its Neumann copy or
// periodic wrap points at (what the reference's ghost fills of matepr and
// matdpr produce).
//
// Ghost values of p and e are never stored: the 7-point stencil maps an
// out-of-range neighbour to the interior cell the reference's ghost copy
// would hold (Neumann: itself; periodic in x/y: the opposite end).
#include "suli_kernels.cuh"

namespace suli {

#define AT(arr, i, j, k) (arr)[g.at((i), (j), (k))]

__device__ __forceinline__ int bmap(int i, int n, bool per)
{
    if (i < 1) return per ? n : 1;
    if (i > n) return per ? 1 : n;
    return i;
}

template <typename T, typename F>
__device__ __forceinline__ T icf(int f, int n, bool periodic, F get)
{
    if (f >= 2 && f <= n) return (get(f) + get(f - 1)) * T(0.5);
    if (periodic) return (get(1) + get(n)) * T(0.5);
    if (f == 1) return (get(2) + get(1)) * T(0.5);
    return (get(n) + get(n - 1)) * T(0.5);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_setup1(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (i > nx || j > ny || k > nz) return;
    const bool px = (c.ccx0 == 0);
    const double dt = c.sc[S_DT];
    const T aux1 = T(dt / (c.dx * c.dx)), aux2 = T(dt / (c.dy * c.dy)), aux3 = T(dt / (c.dz * c.dz));
    const T *rho = c.rho;
    T si0 = aux1 / icf<T>(i, nx, px, [&](int m) { return AT(rho, m, j, k); });
    T si1 = aux1 / icf<T>(i + 1, nx, px, [&](int m) { return AT(rho, m, j, k); });
    T sj0 = aux2 / icf<T>(j, ny, false, [&](int m) { return AT(rho, i, m, k); });
    T sj1 = aux2 / icf<T>(j + 1, ny, false, [&](int m) { return AT(rho, i, m, k); });
    T sk0 = aux3 / icf<T>(k, nz, false, [&](int m) { return AT(rho, i, j, m); });
    T sk1 = aux3 / icf<T>(k + 1, nz, false, [&](int m) { return AT(rho, i, j, m); });
    long long q = g.at(i, j, k);
    c.spi[q] = si0;
    c.spj[q] = sj0;
    c.spk[q] = sk0;
    if (i == nx) c.spi[q + 1] = si1;
    if (j == ny) c.spj[q + g.sx] = sj1;
    if (k == nz) c.spk[q + g.sxy] = sk1;
    c.dpr[q] = si1 + si0 + sj1 + sj0 + sk1 + sk0;
    // right-hand side (:163-183), masked inside an obstacle for ibm_t = 2
    T ua = c.u[q], ub = c.u[q + 1], va = c.v[q], vb = c.v[q + g.sx], wa = c.w[q], wb = c.w[q + g.sxy];
    if (c.obst_t != 0 && c.ibm_t == 2) {
        if (c.obs_lsx[q] >= T(0.)) ua = T(0.);
        if (c.obs_lsx[q + 1] >= T(0.)) ub = T(0.);
        if (c.obs_lsy[q] >= T(0.)) va = T(0.);
        if (c.obs_lsy[q + g.sx] >= T(0.)) vb = T(0.);
        if (c.obs_lsz[q] >= T(0.)) wa = T(0.);
        if (c.obs_lsz[q + g.sxy] >= T(0.)) wb = T(0.);
    }
    c.qpr[q] = (ua - ub) / T(c.dx) + (va - vb) / T(c.dy) + (wa - wb) / T(c.dz);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_setup2(const CaseDev<T> *__restrict__ cs, int ncases, int use_prd1)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (i > nx || j > ny || k > nz) return;
    const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
    const T *D = c.dpr;
    long long q = g.at(i, j, k);
    T Dc = D[q];
    c.spi[q] = c.spi[q] / sqrt(Dc * AT(D, bmap(i - 1, nx, px), j, k));
    c.spj[q] = c.spj[q] / sqrt(Dc * AT(D, i, bmap(j - 1, ny, py), k));
    c.spk[q] = c.spk[q] / sqrt(Dc * AT(D, i, j, bmap(k - 1, nz, false)));
    if (i == nx) c.spi[q + 1] = c.spi[q + 1] / sqrt(AT(D, bmap(nx + 1, nx, px), j, k) * Dc);
    if (j == ny) c.spj[q + g.sx] = c.spj[q + g.sx] / sqrt(AT(D, i, bmap(ny + 1, ny, py), k) * Dc);
    if (k == nz) c.spk[q + g.sxy] = c.spk[q + g.sxy] / sqrt(AT(D, i, j, bmap(nz + 1, nz, false)) * Dc);
    T sD = sqrt(Dc);
    if (use_prd1) c.e[q] = c.prd1[q] * sD;
    c.qpr[q] = c.qpr[q] / sD;
}

// e at a possibly-ghost neighbour: matepr(ghost) = prd1(ghost) * sqrt(matdpr(mapped))
template <typename T>
__device__ __forceinline__ T e_nb(const CaseDev<T> &c, int a, int b, int d, bool px, bool py)
{
    const Geo &g = c.g;
    int ma = bmap(a, g.nx, px), mb = bmap(b, g.ny, py), md = bmap(d, g.nz, false);
    if (ma == a && mb == b && md == d) return AT(c.e, a, b, d);
    return AT(c.prd1, a, b, d) * sqrt(AT(c.dpr, ma, mb, md));
}

template <typename T>
__device__ void cg_start_final(const CaseDev<T> &c, double rr, double bb)
{
    c.sc[S_RR] = rr;
    c.sc[S_RR0] = rr;
    double thr;
    if (c.cg_tol_mode == 1) thr = c.cg_tol * c.cg_tol * bb;
    else thr = c.cg_tol / (double)(c.g.nx * c.g.ny * c.g.nz);
    c.sc[S_THR] = thr;
    c.sc[S_CGITER] = 0.0;
    double replay = c.sc[S_CGREPLAY];
    double active;
    if (replay >= 0.0) active = (0.0 < replay) ? 1.0 : 0.0;
    else active = (fabs(rr) > thr && 0 < c.cg_max) ? 1.0 : 0.0;
    c.sc[S_CGACTIVE] = active;
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_setup3(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
    double rr = 0.0, bb = 0.0;
    if (i <= nx && j <= ny && k <= nz) {
        long long q = g.at(i, j, k);
        T r = c.e[q] - c.spi[q + 1] * e_nb(c, i + 1, j, k, px, py) - c.spi[q] * e_nb(c, i - 1, j, k, px, py) -
              c.spj[q + g.sx] * e_nb(c, i, j + 1, k, px, py) - c.spj[q] * e_nb(c, i, j - 1, k, px, py) -
              c.spk[q + g.sxy] * e_nb(c, i, j, k + 1, px, py) - c.spk[q] * e_nb(c, i, j, k - 1, px, py) - c.qpr[q];
        c.r[q] = r;
        c.p[q] = r;
        rr = (double)r * (double)r;
        bb = (double)c.qpr[q] * (double)c.qpr[q];
    }
    double vals[2] = {rr, bb}, tot[2];
    if (last_block_reduce<T, 2>(c, vals, tot) && tid_lin() == 0) cg_start_final(c, tot[0], tot[1]);
}

// mp = A p, partial p.mp  (9_grad.f90:411-452)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_A(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_CGACTIVE] == 0.0) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
    double pm = 0.0;
    if (i <= nx && j <= ny && k <= nz) {
        const T *__restrict__ p = c.p;
        long long q = g.at(i, j, k);
        T pc = p[q];
        T pxp = (i < nx) ? p[q + 1] : AT(p, bmap(nx + 1, nx, px), j, k);
        T pxm = (i > 1) ? p[q - 1] : AT(p, bmap(0, nx, px), j, k);
        T pyp = (j < ny) ? p[q + g.sx] : AT(p, i, bmap(ny + 1, ny, py), k);
        T pym = (j > 1) ? p[q - g.sx] : AT(p, i, bmap(0, ny, py), k);
        T pzp = (k < nz) ? p[q + g.sxy] : pc;
        T pzm = (k > 1) ? p[q - g.sxy] : pc;
        T m = pc - pxp * c.spi[q + 1] - pxm * c.spi[q] - pyp * c.spj[q + g.sx] - pym * c.spj[q] -
              pzp * c.spk[q + g.sxy] - pzm * c.spk[q];
        c.mp[q] = m;
        pm = (double)pc * (double)m;
    }
    double vals[1] = {pm}, tot[1];
    if (last_block_reduce<T, 1>(c, vals, tot) && tid_lin() == 0) c.sc[S_ALPHA] = c.sc[S_RR] / tot[0];
}

// e -= alpha p, r -= alpha mp, partial r.r  (:458-508)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_B(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_CGACTIVE] == 0.0) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    double rr = 0.0;
    if (i <= g.nx && j <= g.ny && k <= g.nz) {
        long long q = g.at(i, j, k);
        T alpha = T(c.sc[S_ALPHA]);
        c.e[q] = c.e[q] - alpha * c.p[q];
        T r = c.r[q] - alpha * c.mp[q];
        c.r[q] = r;
        rr = (double)r * (double)r;
    }
    double vals[1] = {rr}, tot[1];
    if (last_block_reduce<T, 1>(c, vals, tot) && tid_lin() == 0) {
        double rrn = tot[0];
        c.sc[S_BETA] = rrn / c.sc[S_RR];
        c.sc[S_RR] = rrn;
        double it = c.sc[S_CGITER] + 1.0;
        c.sc[S_CGITER] = it;
        double replay = c.sc[S_CGREPLAY];
        double active;
        if (replay >= 0.0) active = (it < replay) ? 1.0 : 0.0;
        else active = (fabs(rrn) > c.sc[S_THR] && it < c.sc[S_CGMAX]) ? 1.0 : 0.0;
        c.sc[S_CGACTIVE] = active;
    }
}

// p = r + beta p  (:520-526)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_C(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_CGACTIVE] == 0.0) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    long long q = g.at(i, j, k);
    c.p[q] = c.r[q] + T(c.sc[S_BETA]) * c.p[q];
}

// prd1 = e / sqrt(D) on the interior and every ghost mapped to it
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_finish(const CaseDev<T> *__restrict__ cs, int ncases, int from64)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (i > nx || j > ny || k > nz) return;
    const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
    long long q = g.at(i, j, k);
    T val;
    if (from64) val = T(c.e64[q] / sqrt((double)c.dpr[q]));
    else val = c.e[q] / sqrt(c.dpr[q]);
    int xs[3] = {i, -1, -1}, ys[3] = {j, -1, -1}, zs[3] = {k, -1, -1};
    if (bmap(0, nx, px) == i) xs[1] = 0;
    if (bmap(nx + 1, nx, px) == i) xs[2] = nx + 1;
    if (bmap(0, ny, py) == j) ys[1] = 0;
    if (bmap(ny + 1, ny, py) == j) ys[2] = ny + 1;
    if (k == 1) zs[1] = 0;
    if (k == nz) zs[2] = nz + 1;
    for (int a = 0; a < 3; ++a) {
        if (xs[a] < 0) continue;
        for (int b = 0; b < 3; ++b) {
            if (ys[b] < 0) continue;
            for (int d = 0; d < 3; ++d) {
                if (zs[d] < 0) continue;
                AT(c.prd1, xs[a], ys[b], zs[d]) = val;
            }
        }
    }
}

// ---- mixed form: FP32 CG passes inside FP64 iterative refinement -------------
// Each pass: the FP64 residual r64 = A e64 - b (k_cg_true_residual, which also
// tests convergence on its FP64 norm), then an FP32 CG started from x = 0 on
// A x = r (k_cg_A, k_cg_B_pass, k_cg_C) until its residual has dropped by
// 1e3 (or reaches the outer target), then e64 -= x (k_cg_fold).  FP32 CG
// follows FP64 CG iteration for iteration down to ~1e-5 relative residual and
// stalls below, so each pass asks for 1e-3; the FP64 residual of the next
// pass removes the FP32 drift.
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_true_residual(const CaseDev<T> *__restrict__ cs, int ncases, int first)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (!first && c.sc[S_OUTER] < 0.0) return;     // converged earlier
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
    double rr = 0.0, rr32 = 0.0, bb = 0.0;
    if (i <= nx && j <= ny && k <= nz) {
        long long q = g.at(i, j, k);
        const double *e = c.e64;
        auto E = [&](int a, int b2, int d) -> double {
            int ma = bmap(a, nx, px), mb = bmap(b2, ny, py), md = bmap(d, nz, false);
            if (first && !(ma == a && mb == b2 && md == d))
                return (double)AT(c.prd1, a, b2, d) * sqrt((double)AT(c.dpr, ma, mb, md));
            return AT(e, ma, mb, md);
        };
        double r = E(i, j, k) - (double)c.spi[q + 1] * E(i + 1, j, k) - (double)c.spi[q] * E(i - 1, j, k) -
                   (double)c.spj[q + g.sx] * E(i, j + 1, k) - (double)c.spj[q] * E(i, j - 1, k) -
                   (double)c.spk[q + g.sxy] * E(i, j, k + 1) - (double)c.spk[q] * E(i, j, k - 1) - (double)c.qpr[q];
        T r32 = T(r);
        c.r[q] = r32;
        c.p[q] = r32;
        c.e[q] = T(0.);
        rr = r * r;
        rr32 = (double)r32 * (double)r32;
        bb = (double)c.qpr[q] * (double)c.qpr[q];
    }
    double vals[3] = {rr, rr32, bb}, tot[3];
    if (last_block_reduce<T, 3>(c, vals, tot) && tid_lin() == 0) {
        double rrt = tot[0];
        c.sc[S_RRTRUE] = rrt;
        if (first) {
            double thr;
            if (c.cg_tol_mode == 1) thr = c.cg_tol * c.cg_tol * tot[2];
            else thr = c.cg_tol / (double)(nx * ny * nz);
            c.sc[S_THR] = thr;
            c.sc[S_RR0] = rrt;
            c.sc[S_OUTER] = 0.0;
            c.sc[S_CGITER] = 0.0;
        }
        double passes = c.sc[S_OUTER] + 1.0;
        bool conv = !(rrt > c.sc[S_THR]) || c.sc[S_CGITER] >= c.sc[S_CGMAX];
        c.sc[S_RR] = tot[1];
        // inner target: 1e3 reduction, but no further than half the outer target
        c.sc[S_RRREF] = fmax(1e-6 * tot[1], 0.25 * c.sc[S_THR]);
        if (conv) {
            c.sc[S_OUTER] = -passes;           // negative: done after `passes` FP64 residuals
            c.sc[S_CGACTIVE] = 0.0;
        } else {
            c.sc[S_OUTER] = passes;
            c.sc[S_CGACTIVE] = 1.0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_B_rel(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_CGACTIVE] == 0.0) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    double rr = 0.0;
    if (i <= g.nx && j <= g.ny && k <= g.nz) {
        long long q = g.at(i, j, k);
        T alpha = T(c.sc[S_ALPHA]);
        c.e[q] = c.e[q] - alpha * c.p[q];
        T r = c.r[q] - alpha * c.mp[q];
        c.r[q] = r;
        rr = (double)r * (double)r;
    }
    double vals[1] = {rr}, tot[1];
    if (last_block_reduce<T, 1>(c, vals, tot) && tid_lin() == 0) {
        double rrn = tot[0];
        double it = c.sc[S_CGITER] + 1.0;
        c.sc[S_CGITER] = it;
        c.sc[S_BETA] = rrn / c.sc[S_RR];
        c.sc[S_RR] = rrn;
        c.sc[S_CGACTIVE] = (rrn > c.sc[S_RRREF] && it < c.sc[S_CGMAX]) ? 1.0 : 0.0;
    }
}

// e64 += x (the pass's correction) for cases still refining
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_fold(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.sc[S_OUTER] < 0.0) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    long long q = g.at(i, j, k);
    c.e64[q] = c.e64[q] + (double)c.e[q];
}

// e64 = prd1 sqrt(D) on the interior (start of the solve)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_e64_init(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    long long q = g.at(i, j, k);
    c.e64[q] = (double)c.prd1[q] * sqrt((double)c.dpr[q]);
}

// ---- launchers ----------------------------------------------------------------
template <typename T> void launch_cg_setup(const Batch<T> &b, cudaStream_t s)
{
    k_cg_setup1<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_setup2<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 1); count_launch();
    k_cg_setup3<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
template <typename T> void launch_cg_iters(const Batch<T> &b, int n, cudaStream_t s)
{
    for (int q = 0; q < n; ++q) {
        k_cg_A<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
        k_cg_B<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
        k_cg_C<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    }
}
template <typename T> void launch_cg_finish(const Batch<T> &b, cudaStream_t s)
{
    k_cg_finish<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 0); count_launch();
}

// mixed-form pieces
template <typename T> void launch_cg_refine_setup(const Batch<T> &b, cudaStream_t s)
{
    k_cg_setup1<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_setup2<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 0); count_launch();
    k_cg_e64_init<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_true_residual<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 1); count_launch();
}
template <typename T> void launch_cg_refine_inner(const Batch<T> &b, int n, int inner_max, cudaStream_t s)
{
    (void)inner_max;
    for (int q = 0; q < n; ++q) {
        k_cg_A<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
        k_cg_B_rel<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
        k_cg_C<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    }
}
template <typename T> void launch_cg_refine_next(const Batch<T> &b, cudaStream_t s)
{
    k_cg_fold<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_true_residual<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 0); count_launch();
}
template <typename T> void launch_cg_refine_finish(const Batch<T> &b, cudaStream_t s)
{
    k_cg_finish<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 1); count_launch();
}

template void launch_cg_setup<double>(const Batch<double> &, cudaStream_t);
template void launch_cg_iters<double>(const Batch<double> &, int, cudaStream_t);
template void launch_cg_finish<double>(const Batch<double> &, cudaStream_t);
template void launch_cg_setup<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_iters<float>(const Batch<float> &, int, cudaStream_t);
template void launch_cg_finish<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_refine_setup<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_refine_inner<float>(const Batch<float> &, int, int, cudaStream_t);
template void launch_cg_refine_next<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_refine_finish<float>(const Batch<float> &, cudaStream_t);

}  // namespace suli
