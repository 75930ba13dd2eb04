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
// Iteration (the loop of :398-587), over the tiles of the cases still
// iterating only:
//   k_cgi_A      mp = A p and p.mp; the case's last tile forms alpha
//   k_cgi_B      e -= alpha p, r -= alpha mp and r.r; the last tile forms beta,
//                counts the iteration and applies the stop rule; the last
//                case to finish lists the cases still iterating
//   k_cgi_C      p = r + beta p
// Finish: prd1 = e / sqrt(D) (:650-659) on the interior and on every ghost,
// each ghost taking the value of the interior cell its Neumann copy or
// periodic wrap points at (what the reference's ghost fills of matepr and
// matdpr produce).
//
// Ghost values of p and e are never stored: the 7-point stencil maps an
// out-of-range neighbour to the interior cell the reference's ghost copy
// would hold (Neumann: itself; periodic in x/y: the opposite end).
#include "suli_kernels.cuh"

#include <algorithm>

namespace suli {

#define AT(arr, i, j, k) (arr)[g.at((i), (j), (k))]

// iterations of one multigrid-preconditioned FP32 pass at most (a pass that
// stagnates in FP32 hands over to the next FP64 residual)
constexpr int MG_PASS_MAX = 40;

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
// the two cell values icf averages at face f
template <typename T, typename F>
__device__ __forceinline__ void icf_pair(int f, int n, bool periodic, F get, T &a, T &b)
{
    if (f >= 2 && f <= n) { a = get(f); b = get(f - 1); }
    else if (periodic) { a = get(1); b = get(n); }
    else if (f == 1) { a = get(2); b = get(1); }
    else { a = get(n); b = get(n - 1); }
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
    // face densities: interp?_cf of rho, or rho_f1 for the IPA (:103-115)
    const bool ipa = (c.t_press == 2);
    const T r1 = T(c.rho_f1);
    T si0 = aux1 / (ipa ? r1 : icf<T>(i, nx, px, [&](int m) { return AT(rho, m, j, k); }));
    T si1 = aux1 / (ipa ? r1 : icf<T>(i + 1, nx, px, [&](int m) { return AT(rho, m, j, k); }));
    T sj0 = aux2 / (ipa ? r1 : icf<T>(j, ny, false, [&](int m) { return AT(rho, i, m, k); }));
    T sj1 = aux2 / (ipa ? r1 : icf<T>(j + 1, ny, false, [&](int m) { return AT(rho, i, m, k); }));
    T sk0, sk1;
    if (c.dzk) {
        // SuLi-ICdz/9_grad.f90:105,141: dt / (dz(k) dz(k) rho_face), the face
        // density weighted by the spacing
        auto rz = [&](int f) {
            const int ff = f < 2 ? 2 : (f > nz ? nz : f);
            const double a = c.dzk[ff], b = c.dzk[ff - 1];
            return (AT(rho, i, j, ff) * T(a) + AT(rho, i, j, ff - 1) * T(b)) / T(a + b);
        };
        sk0 = T(dt) / (T(c.dzk[k]) * T(c.dzk[k]) * rz(k));
        sk1 = T(dt) / (T(c.dzk[k + 1]) * T(c.dzk[k + 1]) * rz(k + 1));
    } else {
        sk0 = aux3 / (ipa ? r1 : icf<T>(k, nz, false, [&](int m) { return AT(rho, i, j, m); }));
        sk1 = aux3 / (ipa ? r1 : icf<T>(k + 1, nz, false, [&](int m) { return AT(rho, i, j, m); }));
    }
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
    c.qpr[q] = (ua - ub) / T(c.dx) + (va - vb) / T(c.dy) + (wa - wb) / T(c.dzk ? c.dzzk[k] : c.dz);
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

// Mixed form: the operator in FP64 from rho64, built for dt = 1 and kept
// while the density is unchanged (the three RK stages of a step share it).
// The stage's operator is dt times it, so each stage solves the unit system
// L1 p = b / dt for the same pressure, and posdin multiplies the unit face
// factors by dt; the Jacobi scaling and the multigrid preconditioner do not
// see a scalar factor.  op1m forms each face conductance once (the cell's
// low faces, and the high faces on the last cell of a line) with the
// projection's face factor 1 / (h rho_face); op1mb sums the diagonal,
// keeps 1/sqrt(D) in r64 and writes the multigrid's level 0; op2m scales by
// products of 1/sqrt(D).  k_cg_rhs_m then forms each stage's right-hand
// side.  The FP32 iteration uses the rounded scaled coefficients.
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_op1m(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    // the two phases' reciprocal densities, once per block by the same
    // Newton sequence as a face's (a face between two cells of one phase
    // has that phase's density exactly: the mean of two equal values)
    __shared__ double s_ir[2];
    if (tid_lin() == 0) { s_ir[0] = rcp_nr64(c.rho_f1); s_ir[1] = rcp_nr64(c.rho_f2); }
    __syncthreads();
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (i > nx || j > ny || k > nz) return;
    const bool px = (c.ccx0 == 0);
    const double *rho = c.rho64;
    const long long q = g.at(i, j, k);
    const long long b1 = __double_as_longlong(c.rho_f1), b2 = __double_as_longlong(c.rho_f2);
    // per face: the projection's unit factor 1 / (h rho_face), by reciprocal
    // (no FP64 divide), kept for posdin; the operator's coefficient is it / h.
    // Inside a phase (both cells' densities bit-equal to rho_f1 or rho_f2,
    // compared as integers) the face takes the phase's reciprocal: the same
    // bits without the face's FP64 mean and Newton steps on GB300's FP64 pipe
    auto face = [&](double *pf, double *sp, long long qf, double ih, double ra, double rb) {
        const long long ba = __double_as_longlong(ra), bb = __double_as_longlong(rb);
        double ir;
        if (c.t_press == 2) ir = s_ir[0];    // the IPA's operator (9_grad.f90:111-115): rho_f1
        else if (ba == bb && ba == b1) ir = s_ir[0];
        else if (ba == bb && ba == b2) ir = s_ir[1];
        else ir = rcp_nr64((ra + rb) * 0.5);
        const double f = ih * ir;
        pf[qf] = f;
        sp[qf] = f * ih;
    };
    auto facex = [&](long long qf, int fi) {
        double ra, rb;
        icf_pair<double>(fi, nx, px, [&](int m) { return AT(rho, m, j, k); }, ra, rb);
        face(c.pfx64, c.spi64, qf, c.idx, ra, rb);
    };
    auto facey = [&](long long qf, int fj) {
        double ra, rb;
        icf_pair<double>(fj, ny, false, [&](int m) { return AT(rho, i, m, k); }, ra, rb);
        face(c.pfy64, c.spj64, qf, c.idy, ra, rb);
    };
    auto facez = [&](long long qf, int fk) {
        double ra, rb;
        icf_pair<double>(fk, nz, false, [&](int m) { return AT(rho, i, j, m); }, ra, rb);
        face(c.pfz64, c.spk64, qf, c.idz, ra, rb);
    };
    facex(q, i);
    facey(q, j);
    if (c.dzk) {
        // SuLi-ICdz: conductance 1 / (dz(k)^2 rho_face) (9_grad.f90:141), the
        // projection's factor 1 / (dzz(k) rho_face) (10_pos.f90:41), the face
        // density weighted by the spacing
        auto zface = [&](long long qf, int f) {
            const int ff = f < 2 ? 2 : (f > nz ? nz : f);
            const double a = c.dzk[ff], b = c.dzk[ff - 1];
            const double ir = rcp_nr64((AT(rho, i, j, ff) * a + AT(rho, i, j, ff - 1) * b) / (a + b));
            c.pfz64[qf] = c.idzzk[f] * ir;
            c.spk64[qf] = (c.idzk[f] * c.idzk[f]) * ir;
        };
        zface(q, k);
        if (k == nz) zface(q + g.sxy, nz + 1);
    } else {
        facez(q, k);
    }
    if (i == nx) facex(q + 1, nx + 1);
    if (j == ny) facey(q + g.sx, ny + 1);
    if (k == nz && !c.dzk) facez(q + g.sxy, nz + 1);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_op1mb(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (i > nx || j > ny || k > nz) return;
    const long long q = g.at(i, j, k);
    const double si0 = c.spi64[q], si1 = c.spi64[q + 1], sj0 = c.spj64[q], sj1 = c.spj64[q + g.sx];
    const double sk0 = c.spk64[q], sk1 = c.spk64[q + g.sxy];
    const double D = si1 + si0 + sj1 + sj0 + sk1 + sk0;
    c.dpr64[q] = D;
    c.dpr[q] = T(D);
    c.r64[q] = rsqrt(D);
    if (c.nlev > 0) {
        // level 0 of the multigrid preconditioner: the unscaled face
        // conductances, zero on Neumann walls (the wall's ghost copy cancels
        // the face), the wrap face kept on periodic x/y
        const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
        const MgLev<T> &L = c.mg[0];
        const T x0 = (i == 1 && !px) ? T(0) : T(si0), x1 = (i == nx && !px) ? T(0) : T(si1);
        const T y0 = (j == 1 && !py) ? T(0) : T(sj0), y1 = (j == ny && !py) ? T(0) : T(sj1);
        const T z0 = (k == 1) ? T(0) : T(sk0), z1 = (k == nz) ? T(0) : T(sk1);
        L.cx[q] = x0;
        L.cy[q] = y0;
        L.cz[q] = z0;
        if (i == nx) L.cx[q + 1] = x1;
        if (j == ny) L.cy[q + g.sx] = y1;
        if (k == nz) L.cz[q + g.sxy] = z1;
        const T dq = x0 + x1 + y0 + y1 + z0 + z1;
        L.dg[q] = dq;
        L.dgi[q] = (dq > T(0)) ? T(1) / dq : T(0);
    }
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_op2m(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (i > nx || j > ny || k > nz) return;
    const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
    const double *R = c.r64;      // 1/sqrt(D)
    const long long q = g.at(i, j, k);
    const double rc = R[q];
    const double a = c.spi64[q] * (rc * AT(R, bmap(i - 1, nx, px), j, k));
    const double b = c.spj64[q] * (rc * AT(R, i, bmap(j - 1, ny, py), k));
    const double d = c.spk64[q] * (rc * AT(R, i, j, bmap(k - 1, nz, false)));
    c.spi64[q] = a; c.spi[q] = T(a);
    c.spj64[q] = b; c.spj[q] = T(b);
    c.spk64[q] = d; c.spk[q] = T(d);
    if (i == nx) {
        double x = c.spi64[q + 1] * (AT(R, bmap(nx + 1, nx, px), j, k) * rc);
        c.spi64[q + 1] = x; c.spi[q + 1] = T(x);
    }
    if (j == ny) {
        double x = c.spj64[q + g.sx] * (AT(R, i, bmap(ny + 1, ny, py), k) * rc);
        c.spj64[q + g.sx] = x; c.spj[q + g.sx] = T(x);
    }
    if (k == nz) {
        double x = c.spk64[q + g.sxy] * (AT(R, i, j, bmap(nz + 1, nz, false)) * rc);
        c.spk64[q + g.sxy] = x; c.spk[q + g.sxy] = T(x);
    }
}

// A stage's right-hand side on the cached unit operator: the divergence of
// the FP64 velocity masters (the field that posdin corrects) over dt, scaled
// by 1/sqrt(D); the warm start prd1 sqrt(D).  e64 stops holding the last
// pressure here.
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cg_rhs_m(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    if (i == 1 && j == 1 && k == 1) c.sc[S_P64OK] = 0.0;
    const long long q = g.at(i, j, k);
    double ua, ub, va, vb, wa, wb;
    if (c.u64 != nullptr) {
        ua = c.u64[q]; ub = c.u64[q + 1]; va = c.v64[q]; vb = c.v64[q + g.sx]; wa = c.w64[q]; wb = c.w64[q + g.sxy];
    } else {
        ua = c.u[q]; ub = c.u[q + 1]; va = c.v[q]; vb = c.v[q + g.sx]; wa = c.w[q]; wb = c.w[q + g.sxy];
    }
    if (c.obst_t != 0 && c.ibm_t == 2) {
        if (c.obs_lsx[q] >= T(0.)) ua = 0.;
        if (c.obs_lsx[q + 1] >= T(0.)) ub = 0.;
        if (c.obs_lsy[q] >= T(0.)) va = 0.;
        if (c.obs_lsy[q + g.sx] >= T(0.)) vb = 0.;
        if (c.obs_lsz[q] >= T(0.)) wa = 0.;
        if (c.obs_lsz[q + g.sxy] >= T(0.)) wb = 0.;
    }
    const double rc = c.r64[q];
    const double b = ((ua - ub) * c.idx + (va - vb) * c.idy + (wa - wb) * (c.dzk ? c.idzzk[k] : c.idz)) * c.sc[S_IDT];
    const double qs = b * rc;
    c.qpr64[q] = qs;
    c.qpr[q] = T(qs);
    c.e64[q] = (double)c.prd1[q] * (c.dpr64[q] * rc);   // prd1 sqrt(D)
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

// ---- the iteration (the loop of 9_grad.f90:398-587) ----------------------------
// A fixed grid (SMs x resident blocks) walks the chunks (CG_CHUNK tiles) of the
// cases listed in an active-case table (for_active_units); cases that have
// converged are not in the table and cost nothing.  Each thread accumulates
// its cells of a chunk in tile order and the chunk publishes one partial, so
// the reduction order depends on the case alone.  Tables are double-buffered:
// k_cgi_B reads table `in` and, once every listed case has finished its
// reduction, the block that finished last writes the cases still iterating
// to table `out`, which the rest of the iteration and the next k_cgi_A read.

// planes of a column whose loads the streaming kernels issue together (all
// eight in FP32, four in FP64: the registers of five arrays)
template <typename T> constexpr int CG_G = sizeof(T) == 4 ? COL_Z : COL_G;

// mp = A p, partial p.mp (:411-452); the case's last unit forms
// alpha = sc[num] / p.mp (num = S_RR for CG, S_RZ for preconditioned CG).
// Each thread owns a column of COL_Z planes, taken CG_G planes at a time: it
// issues every load of a group (the COL_G + 2 planes of p, the COL_G + 1
// z-face coefficients and the x/y neighbours and coefficients of each plane)
// before any arithmetic, then forms the products; wall and periodic
// neighbours are fixed index offsets and planes past the top are predicated
// off, so nothing branches.
template <typename T>
__global__ void __launch_bounds__(NTHREADS, 2) k_cgi_A(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                       int N, int num)
{
    for_active_units_seg(tab, N, 0, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const Geo &g = c.g;
        const int nx = g.nx, ny = g.ny, nz = g.nz;
        const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
        const T *__restrict__ p = c.p;
        const T *__restrict__ spi = c.spi;
        const T *__restrict__ spj = c.spj;
        const T *__restrict__ spk = c.spk;
        T *__restrict__ mp = c.mp;
        const Column cl = column_of(g, u);
        // 32-bit offsets: a case's box holds fewer than 2^31 elements
        const int sx = (int)g.sx, sxy = (int)g.sxy;
        const int dxp = (cl.i < nx) ? 1 : (px ? -(nx - 1) : 0);
        const int dxm = (cl.i > 1) ? -1 : (px ? (nx - 1) : 0);
        const int dyp = (cl.j < ny) ? sx : (py ? -(ny - 1) * sx : 0);
        const int dym = (cl.j > 1) ? -sx : (py ? (ny - 1) * sx : 0);
        // a thread's products of one unit summed in the storage type (FP32 in
        // the mixed form: the FP64 units of GB300 are a small fraction of its
        // FP32 rate), the block tree and the case total in FP64
        T pm = T(0);
        for (int kb = cl.k0; kb <= cl.k1; kb += CG_G<T>) {
            const int q0 = (int)g.at(cl.i, cl.j, kb);
            const int np = min(CG_G<T>, cl.k1 - kb + 1);
            T pz[CG_G<T> + 2], sk[CG_G<T> + 1];
            T vxp[CG_G<T>], cxp[CG_G<T>], vxm[CG_G<T>], cxm[CG_G<T>], vyp[CG_G<T>], cyp[CG_G<T>], vym[CG_G<T>], cym[CG_G<T>];
#pragma unroll
            for (int t = 0; t < CG_G<T> + 2; ++t) {
                // plane kb-1+t, the Neumann copy at the bottom and top walls
                const int k = min(max(kb - 1 + t, 1), nz);
                pz[t] = p[q0 + (k - kb) * sxy];
            }
#pragma unroll
            for (int t = 0; t < CG_G<T> + 1; ++t) sk[t] = spk[q0 + min(t, np) * sxy];
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                const int q = q0 + min(t, np - 1) * sxy;
                vxp[t] = p[q + dxp]; cxp[t] = spi[q + 1];
                vxm[t] = p[q + dxm]; cxm[t] = spi[q];
                vyp[t] = p[q + dyp]; cyp[t] = spj[q + sx];
                vym[t] = p[q + dym]; cym[t] = spj[q];
            }
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                if (t >= np || !cl.v) continue;
                const T pc = pz[t + 1];
                // the reference's order of operations (9_grad.f90:411-452)
                const T m = pc - vxp[t] * cxp[t] - vxm[t] * cxm[t] - vyp[t] * cyp[t] - vym[t] * cym[t] -
                            pz[t + 2] * sk[t + 1] - pz[t] * sk[t];
                mp[q0 + t * sxy] = m;
                pm += pc * m;
            }
        }
        unit_partial1<T>(c, u, pm);
    }, [&](int id, int cnt) {
        const CaseDev<T> &c = cs[id];
        double tot[1];
        if (seg_reduce<T, 1>(c, cnt, tot) && tid_lin() == 0) c.sc[S_ALPHA] = c.sc[num] / tot[0];
    });
}

// e -= alpha p, r -= alpha mp, partial r.r (:458-508); the case's last unit
// counts the iteration and applies the stop rule:
//   MODE 0  the case's rule (r.r > threshold, iteration cap) or a replayed
//           count; beta = r.r / r.r_old
//   MODE 1  one FP32 pass of the mixed form: r.r above the pass target S_RRREF
//           (at most MG_PASS_MAX iterations when preconditioned, MODE 2)
//   MODE 2  as 1, preconditioned: also writes the V-cycle's right-hand side
//           D^1/2 r (beta comes from r.z, k_pcg_dot)
template <typename T, int MODE>
__global__ void __launch_bounds__(NTHREADS, 2) k_cgi_B(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                    int *__restrict__ out, unsigned *__restrict__ done, int N, int NL)
{
    __shared__ bool compact;
    const int nin = tab[0];
    if (nin == 0) {     // nothing iterates: the next table is empty too
        if (blockIdx.x == 0 && tid_lin() == 0) {
            out[0] = 0;
            for (int s = 0; s < NL; ++s) { out[act_level(N, s)] = 0; out[act_level(N, s) + 1] = 0; }
        }
        return;
    }
    for_active_units_seg(tab, N, 0, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const Geo &g = c.g;
        const T alpha = T(c.sc[S_ALPHA]);
        T *__restrict__ e = c.e;
        T *__restrict__ r = c.r;
        const T *__restrict__ p = c.p;
        const T *__restrict__ mp = c.mp;
        const T *__restrict__ dpr = c.dpr;
        T *__restrict__ f0 = (MODE == 2) ? c.mg[0].f : nullptr;
        const Column cl = column_of(g, u);
        // every load of the column (planes past the top clamped to the last)
        // before any arithmetic; 32-bit offsets (a box holds < 2^31 elements)
        const int q0 = (int)g.at(cl.i, cl.j, cl.k0), sxy = (int)g.sxy, np = cl.k1 - cl.k0 + 1;
        T rr = T(0);
        for (int t0 = 0; t0 < np; t0 += CG_G<T>) {
            T ev[CG_G<T>], pv[CG_G<T>], rv[CG_G<T>], mv[CG_G<T>], dv[CG_G<T>];
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                const int q = q0 + min(t0 + t, np - 1) * sxy;
                ev[t] = e[q]; pv[t] = p[q]; rv[t] = r[q]; mv[t] = mp[q];
                if (MODE == 2) dv[t] = dpr[q];
            }
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                if (t0 + t >= np || !cl.v) continue;
                const int q = q0 + (t0 + t) * sxy;
                const T en = ev[t] - alpha * pv[t];
                const T rn = rv[t] - alpha * mv[t];
                e[q] = en;
                r[q] = rn;
                if (MODE == 2) f0[q] = sqrt(dv[t]) * rn;
                rr += rn * rn;
            }
        }
        unit_partial1<T>(c, u, rr);
    }, [&](int id, int cnt) {
        const CaseDev<T> &c = cs[id];
        double tot[1];
        if (seg_reduce<T, 1>(c, cnt, tot)) {
            if (tid_lin() == 0) {
                double rrn = tot[0];
                double it = c.sc[S_CGITER] + 1.0;
                c.sc[S_CGITER] = it;
                if (MODE != 2) c.sc[S_BETA] = rrn / c.sc[S_RR];
                c.sc[S_RR] = rrn;
                double active;
                if (MODE >= 1) {
                    active = (rrn > c.sc[S_RRREF] && it < c.sc[S_CGMAX] &&
                              (MODE == 1 || it - c.sc[S_PASS0] < (double)MG_PASS_MAX)) ? 1.0 : 0.0;
                } else {
                    double replay = c.sc[S_CGREPLAY];
                    if (replay >= 0.0) active = (it < replay) ? 1.0 : 0.0;
                    else active = (fabs(rrn) > c.sc[S_THR] && it < c.sc[S_CGMAX]) ? 1.0 : 0.0;
                }
                c.sc[S_CGACTIVE] = active;
                __threadfence();
                compact = (atomicAdd(done, 1u) == (unsigned)(nin - 1));
            }
            __syncthreads();
            if (compact) {
                __threadfence();
                build_active_table(cs, N, NL, tab, out);
                if (tid_lin() == 0) *done = 0u;
            }
        }
    });
}

// p = r + beta p (:520-526) over the cases still iterating
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cgi_C(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                    int N)
{
    for_active_units(tab, N, 0, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const Geo &g = c.g;
        const T beta = T(c.sc[S_BETA]);
        const T *__restrict__ r = c.r;
        T *__restrict__ p = c.p;
        const Column cl = column_of(g, u);
        if (!cl.v) return;
        const int q0 = (int)g.at(cl.i, cl.j, cl.k0), sxy = (int)g.sxy, np = cl.k1 - cl.k0 + 1;
        for (int t0 = 0; t0 < np; t0 += CG_G<T>) {
            T rv[CG_G<T>], pv[CG_G<T>];
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                const int q = q0 + min(t0 + t, np - 1) * sxy;
                rv[t] = r[q]; pv[t] = p[q];
            }
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t)
                if (t0 + t < np) p[q0 + (t0 + t) * sxy] = rv[t] + beta * pv[t];
        }
    });
}

// preconditioned CG: r.z with z = D^1/2 z0 (z0 = the V-cycle's result);
// first: start of a pass (beta = 0), else beta = r.z / r.z_old
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_pcg_dot(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                      int N, int first)
{
    for_active_units_seg(tab, N, 0, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const Geo &g = c.g;
        const T *__restrict__ dpr = c.dpr;
        const T *__restrict__ z0 = c.mg[0].z;
        const T *__restrict__ r = c.r;
        const Column cl = column_of(g, u);
        const int q0 = (int)g.at(cl.i, cl.j, cl.k0), sxy = (int)g.sxy, np = cl.k1 - cl.k0 + 1;
        T rz = T(0);
        for (int t0 = 0; t0 < np; t0 += CG_G<T>) {
            T dv[CG_G<T>], zv[CG_G<T>], rv[CG_G<T>];
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                const int q = q0 + min(t0 + t, np - 1) * sxy;
                dv[t] = dpr[q]; zv[t] = z0[q]; rv[t] = r[q];
            }
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                const T z = sqrt(dv[t]) * zv[t];
                if (t0 + t < np && cl.v) rz += z * rv[t];
            }
        }
        unit_partial1<T>(c, u, rz);
    }, [&](int id, int cnt) {
        const CaseDev<T> &c = cs[id];
        double tot[1];
        if (seg_reduce<T, 1>(c, cnt, tot) && tid_lin() == 0) {
            c.sc[S_BETA] = first ? 0.0 : tot[0] / c.sc[S_RZ];
            c.sc[S_RZ] = tot[0];
        }
    });
}

// preconditioned CG: p = D^1/2 z0 + beta p
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_pcg_C(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                    int N)
{
    for_active_units(tab, N, 0, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const Geo &g = c.g;
        const T beta = T(c.sc[S_BETA]);
        const T *__restrict__ dpr = c.dpr;
        const T *__restrict__ z0 = c.mg[0].z;
        T *__restrict__ p = c.p;
        const Column cl = column_of(g, u);
        if (!cl.v) return;
        const int q0 = (int)g.at(cl.i, cl.j, cl.k0), sxy = (int)g.sxy, np = cl.k1 - cl.k0 + 1;
        for (int t0 = 0; t0 < np; t0 += CG_G<T>) {
            T dv[CG_G<T>], zv[CG_G<T>], pv[CG_G<T>];
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t) {
                const int q = q0 + min(t0 + t, np - 1) * sxy;
                dv[t] = dpr[q]; zv[t] = z0[q]; pv[t] = p[q];
            }
#pragma unroll
            for (int t = 0; t < CG_G<T>; ++t)
                if (t0 + t < np) p[q0 + (t0 + t) * sxy] = sqrt(dv[t]) * zv[t] + beta * pv[t];
        }
    });
}

// table `out` := every case of the batch whose S_CGACTIVE is set; clears the
// completion counter (one block)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_cgi_table(const CaseDev<T> *__restrict__ cs, int *__restrict__ out,
                                                        unsigned *__restrict__ done, int N, int NL, int all)
{
    build_active_table<T>(cs, N, NL, nullptr, out, all != 0);
    if (tid_lin() == 0) *done = 0u;
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
    if (from64) {
        // keep the FP64 pressure too (in e64, whose scaled solution is not
        // needed after this): posdin forms its pressure differences from it
        const double p64 = c.e64[q] * c.r64[q];     // r64: 1/sqrt(D) of the cached operator
        c.e64[q] = p64;
        val = T(p64);
        if (i == 1 && j == 1 && k == 1) c.sc[S_P64OK] = 1.0;
    } else {
        val = c.e[q] / sqrt(c.dpr[q]);
    }
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
// Each pass: the FP64 residual b - A e64 (k_cg_true_residual_cols, which
// also tests convergence on its FP64 norm), then an FP32 CG started from
// x = 0 on A x = r (Jacobi-scaled: k_cgi_A, k_cgi_B<1>, k_cgi_C; multigrid-
// preconditioned: the k_pcg kernels around a V-cycle) until its residual has
// dropped by 1e3 (Jacobi) or 1e5 (multigrid), or reaches the outer target,
// then e64 += x (k_cg_fold).  Jacobi-scaled FP32 CG follows FP64 CG
// iteration for iteration down to ~1e-5 relative residual and stalls below;
// the FP64 residual of the next pass removes the FP32 drift.
// A case's scalars after an FP64 residual (thread 0 of its last block):
// convergence, stagnation and the next pass's inner target; bb (the
// right-hand side's r.r) is read on the first residual only
template <typename T>
__device__ void true_residual_update(const CaseDev<T> &c, int first, double rrt, double rr32, double bb)
{
    c.sc[S_RRTRUE] = rrt;
    // stagnation: FP32 passes cannot lower a residual whose worst mode has a
    // condition number near 1/eps(FP32); after three passes that did not
    // halve the best r.r so far (the floor is noisy: against the previous
    // pass a lucky low would restart the count) the case stops
    const double best = first ? rrt : c.sc[S_RRBEST];
    const double stall = first ? 0.0 : ((rrt > 0.5 * best) ? c.sc[S_STALL] + 1.0 : 0.0);
    c.sc[S_STALL] = stall;
    c.sc[S_RRBEST] = fmin(best, rrt);
    if (first) {
        double thr;
        if (c.cg_tol_mode == 1) thr = c.cg_tol * c.cg_tol * bb;
        // (the unit operator's r.r is the stage's over dt)
        else thr = c.cg_tol / ((double)c.g.nx * c.g.ny * c.g.nz) * c.sc[S_IDT];
        c.sc[S_THR] = thr;
        c.sc[S_RR0] = rrt;
        c.sc[S_OUTER] = 0.0;
        c.sc[S_CGITER] = 0.0;
    }
    const double passes = c.sc[S_OUTER] + 1.0;
    const bool stalled = (rrt > c.sc[S_THR]) && stall >= 3.0;
    c.sc[S_STALLED] = stalled ? 1.0 : 0.0;
    const bool conv = !(rrt > c.sc[S_THR]) || c.sc[S_CGITER] >= c.sc[S_CGMAX] || stalled;
    c.sc[S_RR] = rr32;
    // inner target: a residual reduction of 1e3 (Jacobi-scaled passes) or
    // 1e5 (multigrid-preconditioned passes), but no further than half the
    // outer target; a pass also ends after MG_PASS_MAX iterations
    c.sc[S_RRREF] = fmax((c.nlev > 0 ? 1e-10 : 1e-6) * rr32, 0.25 * c.sc[S_THR]);
    c.sc[S_PASS0] = c.sc[S_CGITER];
    if (conv) {
        c.sc[S_OUTER] = -passes;           // negative: done after `passes` FP64 residuals
        c.sc[S_CGACTIVE] = 0.0;
    } else {
        c.sc[S_OUTER] = passes;
        c.sc[S_CGACTIVE] = 1.0;
    }
}

// The FP64 residual of each refinement pass, over column units: a thread
// walks the COL_Z planes of a column, so the FP64 sums cost one block
// reduction per COL_Z cells (with one cell per thread, the per-cell share of
// the FP64 reductions cost more than the residual itself on GB300's FP64
// units).  Every pass applies the operator the passes solve: a Neumann
// neighbour is the cell itself, a periodic one the opposite end.  (The
// reference's first residual takes the ghost values of the warm start,
// prd1 sqrt(D) there; the mixed form starts from the same interior values and
// reads no ghost, which changes only the initial guess.)  first != 0: the
// solve's first residual, with the right-hand side's r.r for the relative
// tolerance; later passes skip the cases that have converged.
template <typename T, int first>
__global__ void __launch_bounds__(NTHREADS, 2) k_cg_true_residual_cols(const CaseDev<T> *__restrict__ cs, int ncases,
                                                                        int nunits)
{
    for (int gu = blockIdx.x; gu < nunits; gu += gridDim.x) {
        int lo = 0, hi = ncases - 1;             // the case of unit gu
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (cs[mid].chunk_begin <= gu) lo = mid; else hi = mid - 1;
        }
        const CaseDev<T> &c = cs[lo];
        if (!first && c.sc[S_OUTER] < 0.0) continue;      // converged (uniform over the block)
        const Geo &g = c.g;
        const int nx = g.nx, ny = g.ny, nz = g.nz;
        const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
        const Column cl = column_of(g, gu - c.chunk_begin);
        const int i = cl.i, j = cl.j;
        const long long sx = g.sx, sxy = g.sxy;
        // neighbour offsets (interior) and, past the grid, the cell a ghost
        // stands for: the opposite end (periodic) or the cell itself (Neumann)
        const bool bxm = i == 1, bxp = i == nx, bym = j == 1, byp = j == ny;
        const long long mxm = px ? (long long)(nx - 1) : 0, mxp = px ? -(long long)(nx - 1) : 0;
        const long long mym = py ? (long long)(ny - 1) * sx : 0, myp = py ? -(long long)(ny - 1) * sx : 0;
        const double *__restrict__ e = c.e64;
        const double *__restrict__ spi = c.spi64;
        const double *__restrict__ spj = c.spj64;
        const double *__restrict__ spk = c.spk64;
        const double *__restrict__ qpr = c.qpr64;
        const T *__restrict__ dpr = c.dpr;
        T *__restrict__ f0 = c.nlev > 0 ? c.mg[0].f : nullptr;
        // the residual's norm from its FP32 rounding, summed per thread in
        // FP32 (a relative 1e-7 on a stopping test; the FP64 pipe is a small
        // fraction of GB300's FP32 rate); the first pass's |b|^2 in FP64
        T rrf = T(0);
        double bb = 0.0;
        if (cl.v) {
            // COL_G planes at a time, every load of a group before any
            // arithmetic; the z-neighbours of the group's planes are the
            // column's planes around it, clamped to the grid (a Neumann wall:
            // the cell itself); 32-bit offsets (a box holds < 2^31 elements)
            const int q0 = (int)g.at(i, j, cl.k0), isx = (int)sx, isxy = (int)sxy, np = cl.k1 - cl.k0 + 1;
            const int dxm = bxm ? (int)mxm : -1, dxp = bxp ? (int)mxp : 1;
            const int dym = bym ? (int)mym : -isx, dyp = byp ? (int)myp : isx;
            for (int kb = 0; kb < np; kb += COL_G) {
                double ec[COL_G + 2], sk[COL_G + 1], exm[COL_G], exq[COL_G], eym[COL_G], eyq[COL_G];
                double sxa[COL_G], sxb[COL_G], sya[COL_G], syb[COL_G], qp[COL_G];
                T dv[COL_G];
#pragma unroll
                for (int t = 0; t < COL_G + 2; ++t) {
                    const int k = min(max(cl.k0 + kb - 1 + t, 1), nz);
                    ec[t] = e[q0 + (k - cl.k0) * isxy];
                }
#pragma unroll
                for (int t = 0; t < COL_G + 1; ++t) sk[t] = spk[q0 + min(kb + t, np) * isxy];
#pragma unroll
                for (int t = 0; t < COL_G; ++t) {
                    const int q = q0 + min(kb + t, np - 1) * isxy;
                    exm[t] = e[q + dxm]; exq[t] = e[q + dxp]; eym[t] = e[q + dym]; eyq[t] = e[q + dyp];
                    sxa[t] = spi[q + 1]; sxb[t] = spi[q]; sya[t] = spj[q + isx]; syb[t] = spj[q];
                    qp[t] = qpr[q];
                    dv[t] = f0 ? dpr[q] : T(0);
                }
#pragma unroll
                for (int t = 0; t < COL_G; ++t) {
                    if (kb + t >= np) continue;
                    const int q = q0 + (kb + t) * isxy;
                    const double r = ec[t + 1] - sxa[t] * exq[t] - sxb[t] * exm[t] - sya[t] * eyq[t] - syb[t] * eym[t] -
                                     sk[t + 1] * ec[t + 2] - sk[t] * ec[t] - qp[t];
                    const T r32 = T(r);
                    c.r[q] = r32;
                    c.p[q] = r32;
                    c.e[q] = T(0.);
                    if (f0) f0[q] = sqrt(dv[t]) * r32;   // V-cycle right-hand side D^1/2 r
                    rrf += r32 * r32;
                    if constexpr (first != 0) bb += qp[t] * qp[t];
                }
            }
        }
        const double rr = (double)rrf, rr32 = rr;
        if constexpr (first != 0) {
            double vals[3] = {rr, rr32, bb}, tot[3];
            if (unit_reduce<T, 3>(c, gu, c.chunk_begin, c.nchunks, vals, tot) && tid_lin() == 0)
                true_residual_update(c, 1, tot[0], tot[1], tot[2]);
        } else {
            double vals[2] = {rr, rr32}, tot[2];
            if (unit_reduce<T, 2>(c, gu, c.chunk_begin, c.nchunks, vals, tot) && tid_lin() == 0)
                true_residual_update(c, 0, tot[0], tot[1], 0.0);
        }
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

// ---- launchers ----------------------------------------------------------------
template <typename T> void launch_cg_setup(const Batch<T> &b, cudaStream_t s)
{
    k_cg_setup1<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_setup2<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 1); count_launch();
    k_cg_setup3<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
// grids of the persistent kernels (each filled to its own occupancy)
template <typename T> struct CgGrids {
    int A, B0, B1, B2, C, dot, pC;
    CgGrids()
    {
        A = occupancy_grid((const void *)k_cgi_A<T>);
        B0 = occupancy_grid((const void *)k_cgi_B<T, 0>);
        B1 = occupancy_grid((const void *)k_cgi_B<T, 1>);
        B2 = occupancy_grid((const void *)k_cgi_B<T, 2>);
        C = occupancy_grid((const void *)k_cgi_C<T>);
        dot = occupancy_grid((const void *)k_pcg_dot<T>);
        pC = occupancy_grid((const void *)k_pcg_C<T>);
    }
};
template <typename T> const CgGrids<T> &cg_grids()
{
    static const CgGrids<T> g;
    return g;
}

template <typename T> const int *cg_table(const Batch<T> &b, int slot)
{
    return b.act + slot * act_stride(b.ncases, b.nlev);
}

template <typename T> void launch_cg_table(const Batch<T> &b, int slot, cudaStream_t s)
{
    k_cgi_table<T><<<1, b.block(), 0, s>>>(b.dcases, b.act + slot * act_stride(b.ncases, b.nlev), b.act_done,
                                           b.ncases, b.nlev, 0);
    count_launch();
}

// Profiling: one launch of a single kernel over every case of the batch,
// on table slot 2 (which the solver never uses).  kernel 0: k_cgi_A (the
// CG matrix-vector product and p.Ap), 1: k_mg_smooth on level 0 (one red
// half-sweep), 2: k_cgi_C (p = r + beta p).  The solver state these touch
// (mp, the level-0 correction, p) is rebuilt by the next pressure solve.
template <typename T> int launch_profile_kernel(const Batch<T> &b, int kernel, int prepare, cudaStream_t s)
{
    int *tab = b.act + 2 * act_stride(b.ncases, b.nlev);
    if (prepare) {
        k_cgi_table<T><<<1, b.block(), 0, s>>>(b.dcases, tab, b.act_done, b.ncases, b.nlev, 1);
        count_launch();
    }
    const CgGrids<T> &G = cg_grids<T>();
    if (kernel == 0) k_cgi_A<T><<<G.A, b.cblock(), 0, s>>>(b.dcases, tab, b.ncases, S_RR);
    else if (kernel == 1) return launch_mg_smooth0<T>(b, tab, 0, s);
    else if (kernel == 2) k_cgi_C<T><<<G.C, b.cblock(), 0, s>>>(b.dcases, tab, b.ncases);
    else if (kernel == 3) return launch_mg_sweep0<T>(b, tab, s);
    else if (kernel == 4) return launch_mg_vcycle_prof<T>(b, tab, s);
    else return -1;
    count_launch();
    return 0;
}

// n iterations starting from table `slot`; returns the slot of the last table
template <typename T> int launch_cg_iters(const Batch<T> &b, int n, int slot, int mode, cudaStream_t s)
{
    const CgGrids<T> &G = cg_grids<T>();
    const int st = act_stride(b.ncases, b.nlev);
    for (int q = 0; q < n; ++q) {
        int *tin = b.act + slot * st, *tout = b.act + (1 - slot) * st;
        k_cgi_A<T><<<G.A, b.cblock(), 0, s>>>(b.dcases, tin, b.ncases, S_RR);
        if (mode == 1) k_cgi_B<T, 1><<<G.B1, b.cblock(), 0, s>>>(b.dcases, tin, tout, b.act_done, b.ncases, b.nlev);
        else k_cgi_B<T, 0><<<G.B0, b.cblock(), 0, s>>>(b.dcases, tin, tout, b.act_done, b.ncases, b.nlev);
        k_cgi_C<T><<<G.C, b.cblock(), 0, s>>>(b.dcases, tout, b.ncases);
        count_launch(3);
        slot = 1 - slot;
    }
    return slot;
}

// start of a preconditioned pass on table `slot` (r and the V-cycle's
// right-hand side written by k_cg_true_residual_cols): z = M r, r.z, p = z
template <typename T> void launch_pcg_start(const Batch<T> &b, int slot, cudaStream_t s)
{
    const CgGrids<T> &G = cg_grids<T>();
    const int *tab = cg_table(b, slot);
    launch_mg_vcycle<T>(b, tab, 0, s);
    k_pcg_dot<T><<<G.dot, b.cblock(), 0, s>>>(b.dcases, tab, b.ncases, 1);
    k_pcg_C<T><<<G.pC, b.cblock(), 0, s>>>(b.dcases, tab, b.ncases);
    count_launch(2);
}

// n preconditioned iterations from table `slot`; returns the current slot
template <typename T> int launch_pcg_iters(const Batch<T> &b, int n, int slot, cudaStream_t s)
{
    const CgGrids<T> &G = cg_grids<T>();
    const int st = act_stride(b.ncases, b.nlev);
    for (int q = 0; q < n; ++q) {
        int *tin = b.act + slot * st, *tout = b.act + (1 - slot) * st;
        k_cgi_A<T><<<G.A, b.cblock(), 0, s>>>(b.dcases, tin, b.ncases, S_RZ);
        k_cgi_B<T, 2><<<G.B2, b.cblock(), 0, s>>>(b.dcases, tin, tout, b.act_done, b.ncases, b.nlev);
        count_launch(2);
        launch_mg_vcycle<T>(b, tout, 0, s);
        k_pcg_dot<T><<<G.dot, b.cblock(), 0, s>>>(b.dcases, tout, b.ncases, 0);
        k_pcg_C<T><<<G.pC, b.cblock(), 0, s>>>(b.dcases, tout, b.ncases);
        count_launch(2);
        slot = 1 - slot;
    }
    return slot;
}

template <typename T> void launch_cg_finish(const Batch<T> &b, cudaStream_t s)
{
    k_cg_finish<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 0); count_launch();
}

// mixed-form pieces
// the unit-dt FP64 operator (kept while the density is unchanged)
template <typename T> void launch_cg_refine_operator(const Batch<T> &b, cudaStream_t s)
{
    k_cg_op1m<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_op1mb<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_op2m<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
// a stage's right-hand side and first FP64 residual
template <typename T> void launch_cg_refine_setup(const Batch<T> &b, cudaStream_t s)
{
    k_cg_rhs_m<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    static const int gR = occupancy_grid((const void *)k_cg_true_residual_cols<T, 1>);
    k_cg_true_residual_cols<T, 1><<<std::min(gR, b.total_units), b.cblock(), 0, s>>>(b.dcases, b.ncases, b.total_units);
    count_launch();
}
template <typename T> void launch_cg_refine_next(const Batch<T> &b, cudaStream_t s)
{
    static const int gR = occupancy_grid((const void *)k_cg_true_residual_cols<T, 0>);
    k_cg_fold<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    k_cg_true_residual_cols<T, 0><<<std::min(gR, b.total_units), b.cblock(), 0, s>>>(b.dcases, b.ncases, b.total_units);
    count_launch();
}
template <typename T> void launch_cg_refine_finish(const Batch<T> &b, cudaStream_t s)
{
    k_cg_finish<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 1); count_launch();
}

template void launch_cg_setup<double>(const Batch<double> &, cudaStream_t);
template void launch_cg_table<double>(const Batch<double> &, int, cudaStream_t);
template int launch_profile_kernel<double>(const Batch<double> &, int, int, cudaStream_t);
template int launch_cg_iters<double>(const Batch<double> &, int, int, int, cudaStream_t);
template void launch_cg_finish<double>(const Batch<double> &, cudaStream_t);
template void launch_cg_setup<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_table<float>(const Batch<float> &, int, cudaStream_t);
template int launch_profile_kernel<float>(const Batch<float> &, int, int, cudaStream_t);
template int launch_cg_iters<float>(const Batch<float> &, int, int, int, cudaStream_t);
template void launch_pcg_start<float>(const Batch<float> &, int, cudaStream_t);
template int launch_pcg_iters<float>(const Batch<float> &, int, int, cudaStream_t);
template void launch_cg_finish<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_refine_operator<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_refine_setup<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_refine_next<float>(const Batch<float> &, cudaStream_t);
template void launch_cg_refine_finish<float>(const Batch<float> &, cudaStream_t);

}  // namespace suli
