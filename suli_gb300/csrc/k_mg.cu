// k_mg.cu -- geometric multigrid V-cycle that preconditions the FP32 CG
// passes of the mixed form (no counterpart in the reference, whose graddin
// is Jacobi-scaled CG, 9_grad.f90:398-587).
//
// The pressure operator of graddin in unscaled form is
//   (L p)_i = sum over the six faces f of cell i of  c_f (p_i - p_nb(f))
// with c_f = dt / (h^2 rho_f) (9_grad.f90:95-148); Neumann walls have c = 0,
// periodic x/y wrap.  The CG iterates on the Jacobi-scaled A = D^-1/2 L D^-1/2,
// so the preconditioner applied to a scaled residual r is
//   z = D^1/2 V(D^1/2 r),   V ~ L^-1 one V-cycle.
//
// Hierarchy: level 0 is the case grid; level l+1 halves every dimension
// (n -> (n+1)/2), coarse cell I owning fine cells 2I-1, 2I.  The coarse
// operator is half the Galerkin product of piecewise-constant aggregation,
// A_c = 1/2 P^T A P: a coarse face conductance is half the sum of the (up to
// four) fine face conductances it covers.  Restriction is P^T (sum of the
// children's residuals), prolongation P (a child takes its parent's value).
// Smoother: red-black Gauss-Seidel, red then black before the coarse
// correction and black then red after it, so the V-cycle is symmetric and
// the preconditioned CG stays a CG.  On a periodic dimension of odd length no
// red-black colouring exists (the wrap neighbours share a colour); there the
// smoother reads the wrap neighbour as zero (keeping the full diagonal) so no
// two cells of one colour couple; residuals and restriction use the full
// operator.
//
// Every kernel runs on a fixed grid over the work units of level l (chunks of
// tiles on level 0, tiles above) of the cases in an active-case table, so
// cases that have converged cost nothing.
#include "suli_kernels.cuh"

#include <cstdlib>

namespace suli {


// one colour of red-black Gauss-Seidel on L z = f; zero != 0: the sweep
// starts from z = 0 (this colour gets f / dg, the other colour 0).  The cells
// of UW tiles are loaded before any is written.
template <typename T>
__global__ void __launch_bounds__(NTHREADS, 4) k_mg_smooth(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                           int N, int l, int color, int zero)
{
    for_active_units(tab, N, l, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const MgLev<T> &L = c.mg[l];
        const Geo &g = L.g;
        const int nx = g.nx, ny = g.ny;
        const long long sx = g.sx, sxy = g.sxy;
        // wrap couplings the smoother keeps (even periodic length, see above);
        // elsewhere a wall neighbour is a ghost of z (never written: zero) and
        // the wall conductance is zero, so the stencil needs no branch
        const bool wx = c.ccx0 == 0 && !(nx & 1) && nx > 1;
        const bool wy = c.ccy0 == 0 && !(ny & 1) && ny > 1;
        const T *z = L.z;
        if (l == 0) {
            // case grid: one column of COL_Z planes per thread, COL_G planes
            // at a time with every load of a group issued before any
            // arithmetic (the z-neighbours of a cell of this colour have the
            // other colour, unchanged by this sweep)
            const Column cl = column_of(g, u);
            const int i = cl.i, j = cl.j;
            // 32-bit offsets: a case's box holds fewer than 2^31 elements
            const int isx = (int)sx, isxy = (int)sxy;
            const int dxm = (wx && i == 1) ? (nx - 1) : -1;
            const int dxp = (wx && i == nx) ? -(nx - 1) : 1;
            const int dym = (wy && j == 1) ? (ny - 1) * isx : -isx;
            const int dyp = (wy && j == ny) ? -(ny - 1) * isx : isx;
            const T *__restrict__ f = L.f;
            const T *__restrict__ dg = L.dg;
            const T *__restrict__ cxa = L.cx;
            const T *__restrict__ cya = L.cy;
            const T *__restrict__ cza = L.cz;
            T *zw = L.z;
            for (int kb = cl.k0; kb <= cl.k1; kb += COL_G) {
                const int q0 = (int)g.at(i, j, kb);
                const int np = min(COL_G, cl.k1 - kb + 1);
                T zz[COL_G + 2], czz[COL_G + 1], fv[COL_G], dv[COL_G];
                T a0[COL_G], a1[COL_G], b0[COL_G], b1[COL_G], za0[COL_G], za1[COL_G], zb0[COL_G], zb1[COL_G];
#pragma unroll
                for (int t = 0; t < COL_G + 2; ++t) zz[t] = z[q0 + (min(t, np + 1) - 1) * isxy];
#pragma unroll
                for (int t = 0; t < COL_G + 1; ++t) czz[t] = cza[q0 + min(t, np) * isxy];
#pragma unroll
                for (int t = 0; t < COL_G; ++t) {
                    const int q = q0 + min(t, np - 1) * isxy;
                    fv[t] = f[q];
                    dv[t] = dg[q];
                    a0[t] = cxa[q]; a1[t] = cxa[q + 1]; b0[t] = cya[q]; b1[t] = cya[q + isx];
                    za0[t] = z[q + dxm]; za1[t] = z[q + dxp]; zb0[t] = z[q + dym]; zb1[t] = z[q + dyp];
                }
#pragma unroll
                for (int t = 0; t < COL_G; ++t) {
                    if (t >= np || !cl.v) continue;
                    const bool mine = ((i + j + kb + t) & 1) == color;
                    const T d = dv[t];
                    T zn;
                    if (zero) {
                        zn = (mine && d > T(0)) ? fv[t] / d : T(0);
                    } else {
                        if (!mine) continue;
                        const T sm = fv[t] + a0[t] * za0[t] + a1[t] * za1[t] + b0[t] * zb0[t] + b1[t] * zb1[t] +
                                     czz[t] * zz[t] + czz[t + 1] * zz[t + 2];
                        zn = (d > T(0)) ? sm / d : T(0);
                    }
                    zw[q0 + t * isxy] = zn;
                }
            }
            return;
        }
        const int t0 = u, t1 = u + 1;
        TileWalk w(t0, L.ntx, L.nty);
        for (int lt = t0; lt < t1; lt += UW) {
            long long q[UW];
            int ci[UW], cj[UW], ck[UW];
            bool v[UW];
            w.next<UW>(lt, t1, g, q, ci, cj, ck, v);
            T zn[UW];
            bool wr[UW];
            if (zero) {
#pragma unroll
                for (int a = 0; a < UW; ++a) {
                    const bool mine = ((ci[a] + cj[a] + ck[a]) & 1) == color;
                    const T d = L.dg[q[a]], fv = L.f[q[a]];
                    zn[a] = (mine && d > T(0)) ? fv / d : T(0);
                    wr[a] = v[a];
                }
            } else {
#pragma unroll
                for (int a = 0; a < UW; ++a) {
                    const int i = ci[a], j = cj[a];
                    const long long qq = q[a];
                    const long long qxm = (wx && i == 1) ? qq + (nx - 1) : qq - 1;
                    const long long qxp = (wx && i == nx) ? qq - (nx - 1) : qq + 1;
                    const long long qym = (wy && j == 1) ? qq + (long long)(ny - 1) * sx : qq - sx;
                    const long long qyp = (wy && j == ny) ? qq - (long long)(ny - 1) * sx : qq + sx;
                    const T d = L.dg[qq];
                    const T s = L.f[qq] + L.cx[qq] * z[qxm] + L.cx[qq + 1] * z[qxp] + L.cy[qq] * z[qym] +
                                L.cy[qq + sx] * z[qyp] + L.cz[qq] * z[qq - sxy] + L.cz[qq + sxy] * z[qq + sxy];
                    zn[a] = (d > T(0)) ? s / d : T(0);
                    wr[a] = v[a] && (((i + j + ck[a]) & 1) == color);
                }
            }
#pragma unroll
            for (int a = 0; a < UW; ++a)
                if (wr[a]) L.z[q[a]] = zn[a];
        }
    });
}

// f(l) = P^T (f - L z)(l-1): the coarse right-hand side, each coarse cell
// summing the residuals of its children
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_mg_restrict(const CaseDev<T> *__restrict__ cs,
                                                          const int *__restrict__ tab, int N, int l)
{
    for_active_units(tab, N, l, [&](int id, int lt) {     // l >= 1: one unit = one tile
        const CaseDev<T> &c = cs[id];
        const MgLev<T> &C = c.mg[l];
        const MgLev<T> &F = c.mg[l - 1];
        int I, J, K;
        tile_cell(C.ntx, C.nty, lt, I, J, K);
        if (I > C.g.nx || J > C.g.ny || K > C.g.nz) return;
        // the full operator (wrap kept on any periodic length); a wall
        // neighbour is a never-written ghost of z (zero) against a zero
        // conductance, and a child beyond an odd fine size is read at a
        // clamped cell and weighted out, so the eight loads need no branch
        const int fx = F.g.nx, fy = F.g.ny, fz = F.g.nz;
        const int sx = (int)F.g.sx, sxy = (int)F.g.sxy;
        const bool wx = c.ccx0 == 0 && fx > 1, wy = c.ccy0 == 0 && fy > 1;
        const T *__restrict__ z = F.z;
        T acc = T(0);
#pragma unroll
        for (int d = 0; d < 8; ++d) {
            const int i0 = 2 * I - 1 + (d & 1), j0 = 2 * J - 1 + ((d >> 1) & 1), k0 = 2 * K - 1 + (d >> 2);
            const bool in = i0 <= fx && j0 <= fy && k0 <= fz;
            const int i = min(i0, fx), j = min(j0, fy), k = min(k0, fz);
            const int q = (int)F.g.at(i, j, k);
            const int qxm = (wx && i == 1) ? q + (fx - 1) : q - 1;
            const int qxp = (wx && i == fx) ? q - (fx - 1) : q + 1;
            const int qym = (wy && j == 1) ? q + (fy - 1) * sx : q - sx;
            const int qyp = (wy && j == fy) ? q - (fy - 1) * sx : q + sx;
            const T r = F.f[q] - F.dg[q] * z[q] + F.cx[q] * z[qxm] + F.cx[q + 1] * z[qxp] + F.cy[q] * z[qym] +
                        F.cy[q + sx] * z[qyp] + F.cz[q] * z[q - sxy] + F.cz[q + sxy] * z[q + sxy];
            acc += in ? r : T(0);
        }
        C.f[C.g.at(I, J, K)] = acc;
    });
}

// z(l) += P z(l+1)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_mg_prolong(const CaseDev<T> *__restrict__ cs,
                                                         const int *__restrict__ tab, int N, int l)
{
    for_active_units(tab, N, l, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const MgLev<T> &F = c.mg[l];
        const MgLev<T> &C = c.mg[l + 1];
        if (l == 0) {
            const Column cl = column_of(F.g, u);
            if (!cl.v) return;
            long long q = F.g.at(cl.i, cl.j, cl.k0);
            for (int k = cl.k0; k <= cl.k1; ++k, q += F.g.sxy)
                F.z[q] += C.z[C.g.at((cl.i + 1) >> 1, (cl.j + 1) >> 1, (k + 1) >> 1)];
            return;
        }
        const int t0 = u, t1 = u + 1;
        TileWalk w(t0, F.ntx, F.nty);
        for (int lt = t0; lt < t1; lt += UW) {
            long long q[UW];
            int ci[UW], cj[UW], ck[UW];
            bool v[UW];
            w.next<UW>(lt, t1, F.g, q, ci, cj, ck, v);
            T zn[UW];
#pragma unroll
            for (int a = 0; a < UW; ++a)
                zn[a] = F.z[q[a]] + C.z[C.g.at((ci[a] + 1) >> 1, (cj[a] + 1) >> 1, (ck[a] + 1) >> 1)];
#pragma unroll
            for (int a = 0; a < UW; ++a)
                if (v[a]) F.z[q[a]] = zn[a];
        }
    });
}

// coarse conductances of level l from level l-1 (all cases of the batch;
// once per pressure solve, after the case grid's level 0 is written)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_mg_coarsen(const CaseDev<T> *__restrict__ cs, int N, int l)
{
    // grid: one block per (case, tile of level l), cases laid out by mg tile
    // offsets computed on the fly (all cases: the launch grid is the sum)
    int b = blockIdx.x, id = 0;
    while (id < N && b >= cs[id].mg[l].ntiles) { b -= cs[id].mg[l].ntiles; ++id; }
    if (id >= N || cs[id].nlev <= l) return;
    const CaseDev<T> &c = cs[id];
    const MgLev<T> &C = c.mg[l];
    const MgLev<T> &F = c.mg[l - 1];
    int I, J, K;
    tile_cell(C.ntx, C.nty, b, I, J, K);
    const int mx = C.g.nx, my = C.g.ny, mz = C.g.nz;
    if (I > mx || J > my || K > mz) return;
    const int fx = F.g.nx, fy = F.g.ny, fz = F.g.nz;
    // fine face index covered by coarse face A (A = 1 .. m+1)
    auto ff = [](int A, int m, int fn) { return (A == m + 1) ? fn + 1 : 2 * A - 1; };
    auto xface = [&](int A) {
        const int fi = ff(A, mx, fx);
        T s = T(0);
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj) {
                const int j = 2 * J - 1 + dj, k = 2 * K - 1 + dk;
                if (j <= fy && k <= fz) s += F.cx[F.g.at(fi, j, k)];
            }
        return T(0.5) * s;
    };
    auto yface = [&](int A) {
        const int fj = ff(A, my, fy);
        T s = T(0);
        for (int dk = 0; dk < 2; ++dk)
            for (int di = 0; di < 2; ++di) {
                const int i = 2 * I - 1 + di, k = 2 * K - 1 + dk;
                if (i <= fx && k <= fz) s += F.cy[F.g.at(i, fj, k)];
            }
        return T(0.5) * s;
    };
    auto zface = [&](int A) {
        const int fk = ff(A, mz, fz);
        T s = T(0);
        for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di) {
                const int i = 2 * I - 1 + di, j = 2 * J - 1 + dj;
                if (i <= fx && j <= fy) s += F.cz[F.g.at(i, j, fk)];
            }
        return T(0.5) * s;
    };
    const Geo &g = C.g;
    const long long q = g.at(I, J, K);
    T x0 = xface(I), x1 = xface(I + 1), y0 = yface(J), y1 = yface(J + 1);
    const T z0 = zface(K), z1 = zface(K + 1);
    // a periodic dimension of one cell: the wrap face joins the cell to itself
    if (c.ccx0 == 0 && mx == 1) x0 = x1 = T(0);
    if (c.ccy0 == 0 && my == 1) y0 = y1 = T(0);
    C.cx[q] = x0;
    C.cy[q] = y0;
    C.cz[q] = z0;
    if (I == mx) C.cx[q + 1] = x1;
    if (J == my) C.cy[q + g.sx] = y1;
    if (K == mz) C.cz[q + g.sxy] = z1;
    // a wrap face joins cells 1 and m: it enters both diagonals; a Neumann
    // wall face is zero already
    C.dg[q] = x0 + x1 + y0 + y1 + z0 + z1;
}

// ---- launchers ---------------------------------------------------------------
template <typename T> void launch_mg_coarsen(const Batch<T> &b, cudaStream_t s)
{
    for (int l = 1; l < b.nlev; ++l) {
        k_mg_coarsen<T><<<b.mg_tiles[l], b.block(), 0, s>>>(b.dcases, b.ncases, l);
        count_launch();
    }
}

// one V-cycle on the cases of table `tab`: level-0 rhs in mg[0].f, result in
// mg[0].z
template <typename T> void launch_mg_vcycle(const Batch<T> &b, const int *tab, int grid, cudaStream_t s)
{
    (void)grid;
    static const int gS = occupancy_grid((const void *)k_mg_smooth<T>);
    static const int gR = occupancy_grid((const void *)k_mg_restrict<T>);
    static const int gP = occupancy_grid((const void *)k_mg_prolong<T>);
    const int N = b.ncases, NL = b.nlev;
    // sweeps before and after the coarse correction: two on every level, the
    // case grid's count settable (SULI_MG_NU0 = 1 or 2) to trade smoothing
    // work on the largest level against iterations
    static const int nu0 = [] {
        const char *e = std::getenv("SULI_MG_NU0");
        return (e && std::atoi(e) == 1) ? 1 : 2;
    }();
    const int ncoarse = 6;
    for (int l = 0; l + 1 < NL; ++l) {
        const int nu = (l == 0) ? nu0 : 2;
        for (int it = 0; it < nu; ++it) {
            k_mg_smooth<T><<<gS, b.cblock(), 0, s>>>(b.dcases, tab, N, l, 0, it == 0);
            k_mg_smooth<T><<<gS, b.cblock(), 0, s>>>(b.dcases, tab, N, l, 1, 0);
        }
        k_mg_restrict<T><<<gR, b.cblock(), 0, s>>>(b.dcases, tab, N, l + 1);
        count_launch(2 * nu + 1);
    }
    for (int it = 0; it < ncoarse; ++it) {
        k_mg_smooth<T><<<gS, b.cblock(), 0, s>>>(b.dcases, tab, N, NL - 1, 0, it == 0);
        k_mg_smooth<T><<<gS, b.cblock(), 0, s>>>(b.dcases, tab, N, NL - 1, 1, 0);
    }
    count_launch(2 * ncoarse);
    for (int l = NL - 2; l >= 0; --l) {
        k_mg_prolong<T><<<gP, b.cblock(), 0, s>>>(b.dcases, tab, N, l);
        const int nu = (l == 0) ? nu0 : 2;
        for (int it = 0; it < nu; ++it) {
            k_mg_smooth<T><<<gS, b.cblock(), 0, s>>>(b.dcases, tab, N, l, 1, 0);
            k_mg_smooth<T><<<gS, b.cblock(), 0, s>>>(b.dcases, tab, N, l, 0, 0);
        }
        count_launch(2 * nu + 1);
    }
}

// profiling: one red half-sweep on level 0 over table `tab`
template <typename T> int launch_mg_smooth0(const Batch<T> &b, const int *tab, int grid, cudaStream_t s)
{
    (void)grid;
    if (b.nlev < 2) return -1;
    static const int gS = occupancy_grid((const void *)k_mg_smooth<T>);
    k_mg_smooth<T><<<gS, b.cblock(), 0, s>>>(b.dcases, tab, b.ncases, 0, 0, 0);
    count_launch();
    return 0;
}
template <> int launch_mg_smooth0<double>(const Batch<double> &, const int *, int, cudaStream_t) { return -1; }

template void launch_mg_coarsen<float>(const Batch<float> &, cudaStream_t);
template int launch_mg_smooth0<float>(const Batch<float> &, const int *, int, cudaStream_t);
template void launch_mg_vcycle<float>(const Batch<float> &, const int *, int, cudaStream_t);

}  // namespace suli
