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
// Every kernel runs on a fixed grid over the work units of level l (column
// units of 32 x 8 cells and COL_Z planes) of the cases in an active-case
// table, so cases that have converged cost nothing.
#include "suli_kernels.cuh"

#include <algorithm>
#include <cstdlib>

namespace suli {


// one colour of red-black Gauss-Seidel on L z = f on level l; zero != 0:
// the sweep starts from z = 0 (this colour gets f / dg, the other colour 0).
// One column of COL_Z planes per thread, COL_G planes at a time with every
// load of a group issued before any arithmetic (the z-neighbours of a cell of
// this colour have the other colour, unchanged by this sweep).
template <typename T>
__global__ void __launch_bounds__(NTHREADS, 4) k_mg_smooth(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                           int N, int l, int color, int zero)
{
    for_active_units(tab, N, l, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const MgLev<T> &L = c.mg[l];
        const Geo &g = L.g;
        const int nx = g.nx, ny = g.ny;
        // wrap couplings the smoother keeps (even periodic length, see above);
        // elsewhere a wall neighbour is a ghost of z (never written: zero) and
        // the wall conductance is zero, so the stencil needs no branch
        const bool wx = c.ccx0 == 0 && !(nx & 1) && nx > 1;
        const bool wy = c.ccy0 == 0 && !(ny & 1) && ny > 1;
        const T *z = L.z;
        const Column cl = column_of(g, u);
        const int i = cl.i, j = cl.j;
        // 32-bit offsets: a case's box holds fewer than 2^31 elements
        const int isx = (int)g.sx, isxy = (int)g.sxy;
        const int dxm = (wx && i == 1) ? (nx - 1) : -1;
        const int dxp = (wx && i == nx) ? -(nx - 1) : 1;
        const int dym = (wy && j == 1) ? (ny - 1) * isx : -isx;
        const int dyp = (wy && j == ny) ? -(ny - 1) * isx : isx;
        const T *__restrict__ f = L.f;
        const T *__restrict__ dgi = L.dgi;
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
                dv[t] = dgi[q];
                a0[t] = cxa[q]; a1[t] = cxa[q + 1]; b0[t] = cya[q]; b1[t] = cya[q + isx];
                za0[t] = z[q + dxm]; za1[t] = z[q + dxp]; zb0[t] = z[q + dym]; zb1[t] = z[q + dyp];
            }
#pragma unroll
            for (int t = 0; t < COL_G; ++t) {
                if (t >= np || !cl.v) continue;
                const bool mine = ((i + j + kb + t) & 1) == color;
                const T di = dv[t];
                T zn;
                if (zero) {
                    zn = mine ? fv[t] * di : T(0);
                } else {
                    if (!mine) continue;
                    const T sm = fv[t] + a0[t] * za0[t] + a1[t] * za1[t] + b0[t] * zb0[t] + b1[t] * zb1[t] +
                                 czz[t] * zz[t] + czz[t + 1] * zz[t + 2];
                    zn = sm * di;
                }
                zw[q0 + t * isxy] = zn;
            }
        }
    });
}

// one half-sweep on level l
template <typename T>
void launch_smooth(const Batch<T> &b, const int *tab, int l, int color, int zero, cudaStream_t s)
{
    static const int g0 = occupancy_grid((const void *)k_mg_smooth<T>);
    k_mg_smooth<T><<<g0, b.cblock(), 0, s>>>(b.dcases, tab, b.ncases, l, color, zero);
}

// One whole red-black sweep of level l in one pass: colour c1, then colour
// c2 = 1 - c1, reading z from buffer `src` and writing every cell of the
// grid to buffer `dst` (0: z, 1: z2; src != dst unless zero, the sweep from
// z = 0, which reads no z).  A block walks a column unit plane by
// plane.  For each plane it computes the c1 values on the unit's 34 x 10
// footprint (the unit and a one-cell ring, wrap neighbours resolved to the
// cells they stand for) into a three-plane ring in shared memory, and then
// updates the c2 cells of the plane below from those values.  The ring cells
// are computed by both blocks that need them, from the same inputs, so the
// two half-sweeps need one trip through memory instead of two; the results
// are the two half-sweep launches' (same operands, same order).  The units
// are dealt to the blocks round-robin (for_active_units_rr), so a unit's x-
// and y-neighbours are swept at the same time by other blocks and the halo
// rows they share come from DRAM once and hit in L2 for the other.
//
// The inputs of a plane (z over the footprint and one more cell around it,
// f, dg and the three conductances over the footprint) are staged in shared
// memory by 16-byte asynchronous copies (cp.async), whole 40-float row
// segments, in a ring of SW_NS planes issued three planes ahead of the one
// being computed, so the loads of later planes are in flight while a plane
// is computed.  Segments outside the case's box are not copied; only cells
// outside the grid (never used) would read them.  Cells whose stencil
// crosses a periodic wrap read their operands from global memory instead.
constexpr int SW_X = COL_X + 2, SW_Y = COL_Y + 2, SW_N = SW_X * SW_Y;
constexpr int SW_R = 40;                     // floats per staged row segment (10 x 16 B)
constexpr int SW_ZR = COL_Y + 4;             // rows of z (j0-2 .. j0+9)
constexpr int SW_CR = COL_Y + 2;             // rows of f, dg, cx, cz (j0-1 .. j0+8)
constexpr int SW_YR = COL_Y + 3;             // rows of cy (j0-1 .. j0+9)
constexpr int SW_OZ = 0, SW_OF = SW_OZ + SW_ZR * SW_R, SW_OD = SW_OF + SW_CR * SW_R, SW_OX = SW_OD + SW_CR * SW_R,
              SW_OY = SW_OX + SW_CR * SW_R, SW_OC = SW_OY + SW_YR * SW_R, SW_STAGE = SW_OC + SW_CR * SW_R;
constexpr int SW_CHUNKS = SW_STAGE / 4;      // 16-byte copies per plane
constexpr int SW_NS = 5;                     // planes in the staging ring
constexpr int SW_SLOTS = (SW_CHUNKS + NTHREADS - 1) / NTHREADS;
constexpr size_t SW_SMEM = (size_t)SW_NS * SW_STAGE * 4;   // dynamic shared memory (T = float)

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <typename T>
__global__ void __launch_bounds__(NTHREADS, 4) k_mg_sweep(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                          int N, int l, int c1, int zero, int src, int dst)
{
    static_assert(sizeof(T) == 4, "the staged sweep is the FP32 smoother");
    extern __shared__ __align__(16) unsigned char sw_dyn[];
    T *stg = reinterpret_cast<T *>(sw_dyn);
    __shared__ T ring[3][SW_N];
    const int t = tid_lin();
    for_active_units_rr(tab, N, l, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const MgLev<T> &L = c.mg[l];
        const Geo &g = L.g;
        const int nx = g.nx, ny = g.ny, nz = g.nz;
        const int isx = (int)g.sx, isxy = (int)g.sxy;
        const bool wx = c.ccx0 == 0 && !(nx & 1) && nx > 1;
        const bool wy = c.ccy0 == 0 && !(ny & 1) && ny > 1;
        const T *__restrict__ zs = src ? L.z2 : L.z;
        T *__restrict__ zd = dst ? L.z2 : L.z;
        const int ux = (nx + COL_X - 1) / COL_X, uy = (ny + COL_Y - 1) / COL_Y;
        const int i0 = 1 + (u % ux) * COL_X, j0 = 1 + ((u / ux) % uy) * COL_Y;
        const int k0 = 1 + (u / (ux * uy)) * COL_Z, k1 = min(nz, k0 + COL_Z - 1);
        const int c2 = 1 - c1;
        const int X0 = i0 - 5;                   // x of a staged row's first float (a multiple of 4)
        // this thread's copy slots: shared offset in a stage, source address
        // of plane k0 - 2 (advanced one plane per issue), kind; a segment
        // outside the box in x or y is never copied
        // (smask: bit t set when the slot copies in a plane of type t -- 0 the
        // unit's first plane k0 - 2 (z only), 1 its last k1 + 2 (z and cz),
        // 2 any other; a slot outside the box or the stage copies in none)
        int so[SW_SLOTS], smask[SW_SLOTS];
        const T *gp[SW_SLOTS];
#pragma unroll
        for (int s = 0; s < SW_SLOTS; ++s) {
            const int ch = t + s * NTHREADS;
            const int e = ch * 4;                // float offset in the stage
            int base, rows0, kind;               // kind 0: z, 1: f, dgi, cx, cy, 2: cz
            const T *arr;
            if (e < SW_OF) { base = SW_OZ; rows0 = j0 - 2; arr = zs; kind = 0; }
            else if (e < SW_OD) { base = SW_OF; rows0 = j0 - 1; arr = L.f; kind = 1; }
            else if (e < SW_OX) { base = SW_OD; rows0 = j0 - 1; arr = L.dgi; kind = 1; }
            else if (e < SW_OY) { base = SW_OX; rows0 = j0 - 1; arr = L.cx; kind = 1; }
            else if (e < SW_OC) { base = SW_OY; rows0 = j0 - 1; arr = L.cy; kind = 1; }
            else { base = SW_OC; rows0 = j0 - 1; arr = L.cz; kind = 2; }
            const int r = (e - base) / SW_R, h = (e - base) % SW_R;
            const int x = X0 + h, y = rows0 + r;
            so[s] = e;
            const bool sv = ch < SW_CHUNKS && x >= 0 && x + 4 <= isx && y >= 0 && y <= ny + 1 && !(zero && kind == 0);
            smask[s] = sv ? (kind == 0 ? 7 : (kind == 2 ? 6 : 4)) : 0;
            gp[s] = arr + (x + isx * y) + (long long)isxy * (k0 - 2);
        }
        // plane p's copies into stage `st`: of plane k0 - 2 only z is read,
        // of k1 + 2 only z and cz, nothing above k1 + 2
        auto issue = [&](int p, int st) {
            if (p >= 0 && p <= nz + 1 && p <= k1 + 2) {
                T *S = stg + st * SW_STAGE;
                const int bit = (p == k0 - 2) ? 1 : (p == k1 + 2) ? 2 : 4;
#pragma unroll
                for (int s = 0; s < SW_SLOTS; ++s)
                    if (smask[s] & bit) cp_async16(S + so[s], gp[s]);
            }
#pragma unroll
            for (int s = 0; s < SW_SLOTS; ++s) gp[s] += isxy;
            cp_async_commit();
        };
        auto wrap5 = [](int s) { return s >= SW_NS ? s - SW_NS : s; };
        // this thread's first-colour footprint position (t < 170): row pj,
        // column 2 pm + b with b the plane's parity choice; both choices
        // resolved here (ring index, staged offset, in the grid, wrapped)
        const bool pt = t < SW_Y * (SW_X / 2);
        const int pj = t / (SW_X / 2), pm = t % (SW_X / 2);
        const int lj = j0 - 1 + pj;
        int rj = lj;
        if (wy && lj == 0) rj = ny;
        if (wy && lj == ny + 1) rj = 1;
        const bool pvy = pt && rj >= 1 && rj <= ny;
        const bool pwy = wy && (lj <= 1 || lj >= ny);
        rj = max(1, min(rj, ny));
        // flags of choice b in bit b; the offsets of choice 1 are those of
        // choice 0 plus one
        int pvb = 0, pwb = 0, pq0 = 0, pq1 = 0;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int li = i0 - 1 + 2 * pm + b;
            int ri = li;
            if (wx && li == 0) ri = nx;
            if (wx && li == nx + 1) ri = 1;
            if (pvy && ri >= 1 && ri <= nx) pvb |= 1 << b;
            if (pwy || (wx && (li <= 1 || li >= nx))) pwb |= 1 << b;
            ri = max(1, min(ri, nx));
            (b ? pq1 : pq0) = ri + isx * rj;
        }
        const int pr0 = pj * SW_X + 2 * pm, pe0 = pj * SW_R + 2 * pm + 4;
        // this thread's own cell
        const int oi = i0 + (t & (COL_X - 1)), oj = j0 + t / COL_X;
        const bool ov = oi <= nx && oj <= ny;
        const int op = (t & (COL_X - 1)) + 1 + SW_X * (t / COL_X + 1);
        const int os = (t / COL_X + 1) * SW_R + (t & (COL_X - 1)) + 5;
        T *zo = zd + (min(oi, nx) + isx * min(oj, ny)) + (long long)isxy * k0;
        __syncthreads();          // the previous unit's stages and ring are consumed
#pragma unroll 1
        for (int p = k0 - 2; p <= k0 + 1; ++p) issue(p, p - (k0 - 2));
        int sm1 = 0;              // stage of plane kk - 1
        int rr = 2;               // ring slot of plane kk
#pragma unroll 1
        for (int kk = k0 - 1; kk <= k1 + 1; ++kk) {
            cp_async_wait<1>();   // planes up to kk + 1 have landed (kk + 2 may be in flight)
            __syncthreads();
            issue(kk + 3, wrap5(sm1 + 4));   // into the stage of plane kk - 2, read for the last time above
            const T *Sm = stg + sm1 * SW_STAGE, *S0 = stg + wrap5(sm1 + 1) * SW_STAGE,
                    *Sp = stg + wrap5(sm1 + 2) * SW_STAGE;
            // c1 values of plane kk on the footprint (zero outside the grid;
            // the c2 positions of the ring are never read)
            T *R = ring[rr];
            if (pt) {
                const int b = (c1 + lj + kk) & 1;                 // i0 - 1 is even
                T zn = T(0);
                if (((pvb >> b) & 1) && kk >= 1 && kk <= nz) {
                    T fv, di, a0, a1, b0, b1, e0, e1, za0 = T(0), za1 = T(0), zb0 = T(0), zb1 = T(0), zc0 = T(0), zc1 = T(0);
                    if ((pwb >> b) & 1) {
                        const int q = (b ? pq1 : pq0) + isxy * kk;
                        const int ri = q % isx;
                        const int pxm = (wx && ri == 1) ? (nx - 1) : -1;
                        const int pxp = (wx && ri == nx) ? -(nx - 1) : 1;
                        const int pym = (wy && rj == 1) ? (ny - 1) * isx : -isx;
                        const int pyp = (wy && rj == ny) ? -(ny - 1) * isx : isx;
                        fv = L.f[q]; di = L.dgi[q];
                        a0 = L.cx[q]; a1 = L.cx[q + 1]; b0 = L.cy[q]; b1 = L.cy[q + isx]; e0 = L.cz[q]; e1 = L.cz[q + isxy];
                        if (!zero) {
                            za0 = zs[q + pxm]; za1 = zs[q + pxp]; zb0 = zs[q + pym]; zb1 = zs[q + pyp];
                            zc0 = zs[q - isxy]; zc1 = zs[q + isxy];
                        }
                    } else {
                        const int e = pe0 + b;
                        fv = S0[SW_OF + e]; di = S0[SW_OD + e];
                        a0 = S0[SW_OX + e]; a1 = S0[SW_OX + e + 1]; b0 = S0[SW_OY + e]; b1 = S0[SW_OY + e + SW_R];
                        e0 = S0[SW_OC + e]; e1 = Sp[SW_OC + e];
                        if (!zero) {
                            const int ez = e + SW_R;     // z rows start one row lower
                            za0 = S0[SW_OZ + ez - 1]; za1 = S0[SW_OZ + ez + 1];
                            zb0 = S0[SW_OZ + ez - SW_R]; zb1 = S0[SW_OZ + ez + SW_R];
                            zc0 = Sm[SW_OZ + ez]; zc1 = Sp[SW_OZ + ez];
                        }
                    }
                    if (zero) {
                        zn = fv * di;
                    } else {
                        const T sm = fv + a0 * za0 + a1 * za1 + b0 * zb0 + b1 * zb1 + e0 * zc0 + e1 * zc1;
                        zn = sm * di;
                    }
                }
                R[pr0 + b] = zn;
            }
            __syncthreads();
            // plane kb = kk - 1: c2 cells from the ring, c1 cells copied out
            const int kb = kk - 1;
            if (kb >= k0) {
                if (ov) {
                    // ring slots of planes kb - 1 (= kk - 2) and kb (= kk - 1);
                    // both colours evaluate the stencil (its operands are in
                    // place either way), the first colour keeps its ring value
                    const T *Rm = ring[rr == 2 ? 0 : rr + 1], *R0 = ring[rr == 0 ? 2 : rr - 1], *Rp = R;
                    const T sm = Sm[SW_OF + os] + Sm[SW_OX + os] * R0[op - 1] + Sm[SW_OX + os + 1] * R0[op + 1] +
                                 Sm[SW_OY + os] * R0[op - SW_X] + Sm[SW_OY + os + SW_R] * R0[op + SW_X] +
                                 Sm[SW_OC + os] * Rm[op] + S0[SW_OC + os] * Rp[op];
                    *zo = (((oi + oj + kb) & 1) == c2) ? sm * Sm[SW_OD + os] : R0[op];
                }
                zo += isxy;
            }
            sm1 = wrap5(sm1 + 1);
            rr = (rr == 2) ? 0 : rr + 1;
        }
        cp_async_wait<0>();       // no copy of this unit is left in flight
    });
}

// the one-pass sweep's grid: its dynamic shared memory opted in, every SM
// filled to the occupancy that memory allows
template <typename T> int sweep_grid(const Batch<T> &b)
{
    static const int full = [] {
        cudaFuncSetAttribute((const void *)k_mg_sweep<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SW_SMEM);
        return occupancy_grid((const void *)k_mg_sweep<T>, SW_SMEM);
    }();
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    // the autotuner may run fewer blocks per SM than the occupancy limit
    const int per = b.tune.sweep_blocks_per_sm;
    return (per > 0 && per * sms < full) ? per * sms : full;
}

// f(l) = P^T (f - L z)(l-1): the coarse right-hand side, each coarse cell
// summing the residuals of its children; one column unit of level l per
// unit of work (each thread a column of up to COL_Z coarse cells)
template <typename T>
__global__ void __launch_bounds__(NTHREADS, 2) k_mg_restrict(const CaseDev<T> *__restrict__ cs,
                                                          const int *__restrict__ tab, int N, int l)
{
    for_active_units(tab, N, l, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const MgLev<T> &C = c.mg[l];
        const MgLev<T> &F = c.mg[l - 1];
        const Column cl = column_of(C.g, u);
        if (!cl.v) return;
        const int I = cl.i, J = cl.j;
        // the full operator (wrap kept on any periodic length); a wall
        // neighbour is a never-written ghost of z (zero) against a zero
        // conductance, and a child beyond an odd fine size is read at a
        // clamped cell and weighted out, so the eight loads need no branch
        const int fx = F.g.nx, fy = F.g.ny, fz = F.g.nz;
        const int sx = (int)F.g.sx, sxy = (int)F.g.sxy;
        const bool wx = c.ccx0 == 0 && fx > 1, wy = c.ccy0 == 0 && fy > 1;
        const T *__restrict__ z = F.z;
        const T *__restrict__ ff = F.f;
        const T *__restrict__ fdg = F.dg;
        const T *__restrict__ fcx = F.cx;
        const T *__restrict__ fcy = F.cy;
        const T *__restrict__ fcz = F.cz;
        T *__restrict__ cf = C.f;
#pragma unroll 2
        for (int K = cl.k0; K <= cl.k1; ++K) {
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
                const T r = ff[q] - fdg[q] * z[q] + fcx[q] * z[qxm] + fcx[q + 1] * z[qxp] + fcy[q] * z[qym] +
                            fcy[q + sx] * z[qyp] + fcz[q] * z[q - sxy] + fcz[q + sxy] * z[q + sxy];
                acc += in ? r : T(0);
            }
            cf[C.g.at(I, J, K)] = acc;
        }
    });
}

// z(l) += P z(l+1); with to2 the sum goes to z2 (z unchanged)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_mg_prolong(const CaseDev<T> *__restrict__ cs,
                                                         const int *__restrict__ tab, int N, int l, int to2)
{
    for_active_units(tab, N, l, [&](int id, int u) {
        const CaseDev<T> &c = cs[id];
        const MgLev<T> &F = c.mg[l];
        const MgLev<T> &C = c.mg[l + 1];
        const Column cl = column_of(F.g, u);
        if (!cl.v) return;
        T *__restrict__ out = to2 ? F.z2 : F.z;
        const T *__restrict__ zf = F.z;
        const T *__restrict__ zc = C.z;
        // every load of the column before any store (planes past the top
        // clamped to the last); 32-bit offsets
        const int q0 = (int)F.g.at(cl.i, cl.j, cl.k0), sxy = (int)F.g.sxy, np = cl.k1 - cl.k0 + 1;
        const int c0 = (int)C.g.at((cl.i + 1) >> 1, (cl.j + 1) >> 1, 0), csxy = (int)C.g.sxy;
        T fv[COL_Z], cv[COL_Z];
#pragma unroll
        for (int t = 0; t < COL_Z; ++t) {
            const int k = cl.k0 + min(t, np - 1);
            fv[t] = zf[q0 + min(t, np - 1) * sxy];
            cv[t] = zc[c0 + ((k + 1) >> 1) * csxy];
        }
#pragma unroll
        for (int t = 0; t < COL_Z; ++t)
            if (t < np) out[q0 + t * sxy] = fv[t] + cv[t];
    });
}

// The coarse end of the V-cycle in one thread block per active case: from
// level lc (small enough for one SM) down to the coarsest and back, each
// half-sweep, restriction and prolongation a block-wide loop over the
// level's cells with a barrier between them (a block's global writes are
// visible to the block after __syncthreads).  Per cell the same arithmetic
// as k_mg_smooth's tile path, k_mg_restrict and k_mg_prolong, in the same
// order of phases; it replaces about ten launches per level.
template <typename T>
__device__ __forceinline__ void mg_cell_ijk(const Geo &g, int t, int &i, int &j, int &k)
{
    i = 1 + t % g.nx;
    const int r = t / g.nx;
    j = 1 + r % g.ny;
    k = 1 + r / g.ny;
}

template <typename T>
__device__ void mg_block_smooth(const CaseDev<T> &c, const MgLev<T> &L, int color, int zero)
{
    const Geo &g = L.g;
    const int nx = g.nx, ny = g.ny, n = nx * ny * g.nz;
    const long long sx = g.sx, sxy = g.sxy;
    const bool wx = c.ccx0 == 0 && !(nx & 1) && nx > 1;
    const bool wy = c.ccy0 == 0 && !(ny & 1) && ny > 1;
    const T *z = L.z;
    for (int t = threadIdx.x + blockDim.x * threadIdx.y; t < n; t += blockDim.x * blockDim.y) {
        int i, j, k;
        mg_cell_ijk<T>(g, t, i, j, k);
        const long long qq = g.at(i, j, k);
        const bool mine = ((i + j + k) & 1) == color;
        if (zero) {
            const T di = L.dgi[qq], fv = L.f[qq];
            L.z[qq] = mine ? fv * di : T(0);
            continue;
        }
        if (!mine) continue;
        const long long qxm = (wx && i == 1) ? qq + (nx - 1) : qq - 1;
        const long long qxp = (wx && i == nx) ? qq - (nx - 1) : qq + 1;
        const long long qym = (wy && j == 1) ? qq + (long long)(ny - 1) * sx : qq - sx;
        const long long qyp = (wy && j == ny) ? qq - (long long)(ny - 1) * sx : qq + sx;
        const T di = L.dgi[qq];
        const T sm = L.f[qq] + L.cx[qq] * z[qxm] + L.cx[qq + 1] * z[qxp] + L.cy[qq] * z[qym] + L.cy[qq + sx] * z[qyp] +
                     L.cz[qq] * z[qq - sxy] + L.cz[qq + sxy] * z[qq + sxy];
        L.z[qq] = sm * di;
    }
    __syncthreads();
}

template <typename T>
__device__ void mg_block_restrict(const CaseDev<T> &c, const MgLev<T> &F, const MgLev<T> &C)
{
    const int fx = F.g.nx, fy = F.g.ny, fz = F.g.nz;
    const int sx = (int)F.g.sx, sxy = (int)F.g.sxy;
    const bool wx = c.ccx0 == 0 && fx > 1, wy = c.ccy0 == 0 && fy > 1;
    const T *__restrict__ z = F.z;
    const int n = C.g.nx * C.g.ny * C.g.nz;
    for (int t = threadIdx.x + blockDim.x * threadIdx.y; t < n; t += blockDim.x * blockDim.y) {
        int I, J, K;
        mg_cell_ijk<T>(C.g, t, I, J, K);
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
    }
    __syncthreads();
}

template <typename T>
__device__ void mg_block_prolong(const MgLev<T> &F, const MgLev<T> &C)
{
    const int n = F.g.nx * F.g.ny * F.g.nz;
    for (int t = threadIdx.x + blockDim.x * threadIdx.y; t < n; t += blockDim.x * blockDim.y) {
        int i, j, k;
        mg_cell_ijk<T>(F.g, t, i, j, k);
        const long long q = F.g.at(i, j, k);
        F.z[q] = F.z[q] + C.z[C.g.at((i + 1) >> 1, (j + 1) >> 1, (k + 1) >> 1)];
    }
    __syncthreads();
}

constexpr int MG_COARSE_THREADS = 1024;   // per block: a few cells per thread on a 16k-cell level

template <typename T>
__global__ void __launch_bounds__(MG_COARSE_THREADS) k_mg_coarse(const CaseDev<T> *__restrict__ cs, const int *__restrict__ tab,
                                                        int lc, int NL, int nuc, int ncoarse)
{
    const int n = tab[0];
    for (int a = blockIdx.x; a < n; a += gridDim.x) {
        const CaseDev<T> &c = cs[tab[1 + a]];
        for (int l = lc; l + 1 < NL; ++l) {
            for (int it = 0; it < nuc; ++it) {
                mg_block_smooth<T>(c, c.mg[l], 0, it == 0);
                mg_block_smooth<T>(c, c.mg[l], 1, 0);
            }
            mg_block_restrict<T>(c, c.mg[l], c.mg[l + 1]);
        }
        for (int it = 0; it < ncoarse; ++it) {
            mg_block_smooth<T>(c, c.mg[NL - 1], 0, it == 0);
            mg_block_smooth<T>(c, c.mg[NL - 1], 1, 0);
        }
        for (int l = NL - 2; l >= lc; --l) {
            mg_block_prolong<T>(c.mg[l], c.mg[l + 1]);
            for (int it = 0; it < nuc; ++it) {
                mg_block_smooth<T>(c, c.mg[l], 1, 0);
                mg_block_smooth<T>(c, c.mg[l], 0, 0);
            }
        }
    }
}

// first level handled by k_mg_coarse: the first whose largest grid over the
// batch has at most b.tune.mg_block_cells cells (the autotuner's choice,
// default 16384; 0: none, every level by whole-grid launches); at least 1, at
// most NL (none)
template <typename T> int mg_block_level(const Batch<T> &b)
{
    const int limit = b.tune.mg_block_cells;
    if (limit <= 0) return b.nlev;
    for (int l = 1; l < b.nlev; ++l) {
        long long mx = 0;
        for (int c = 0; c < b.ncases; ++c) {
            const Geo &g = b.hcases[c].mg[l].g;
            mx = std::max<long long>(mx, (long long)g.nx * g.ny * g.nz);
        }
        if (mx <= limit) return l;
    }
    return b.nlev;
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
    const T dq = x0 + x1 + y0 + y1 + z0 + z1;
    C.dg[q] = dq;
    C.dgi[q] = (dq > T(0)) ? T(1) / dq : T(0);
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
    // the same for the coarser levels (SULI_MG_NUC = 1 or 2)
    static const int nuc = [] {
        const char *e = std::getenv("SULI_MG_NUC");
        return (e && std::atoi(e) == 1) ? 1 : 2;
    }();
    // the sweeps of the levels smoothed by launches as one-pass whole
    // sweeps, or (SULI_MG_FUSED=0) as two half-sweep launches each: the same
    // arithmetic
    const char *fe = std::getenv("SULI_MG_FUSED");
    const bool fused = !(fe && std::atoi(fe) == 0);
    const int gW = sweep_grid<T>(b);
    const int ncoarse = 6;
    // levels lc.. in one block per case (k_mg_coarse), the finer ones by
    // whole-grid launches
    const int lc = mg_block_level<T>(b);
    const int ldown = (lc < NL) ? lc : NL - 1;    // levels smoothed by launches before the coarse end
    for (int l = 0; l < ldown; ++l) {
        const int nu = (l == 0) ? nu0 : nuc;
        if (fused) {
            // the buffers alternate so that the last sweep writes z
            for (int it = 0; it < nu; ++it) {
                const int dst = (nu - 1 - it) & 1;
                k_mg_sweep<T><<<gW, b.cblock(), SW_SMEM, s>>>(b.dcases, tab, N, l, 0, it == 0, 1 - dst, dst);
            }
            k_mg_restrict<T><<<gR, b.cblock(), 0, s>>>(b.dcases, tab, N, l + 1);
            count_launch(nu + 1);
            continue;
        }
        for (int it = 0; it < nu; ++it) {
            launch_smooth<T>(b, tab, l, 0, it == 0, s);
            launch_smooth<T>(b, tab, l, 1, 0, s);
        }
        k_mg_restrict<T><<<gR, b.cblock(), 0, s>>>(b.dcases, tab, N, l + 1);
        count_launch(2 * nu + 1);
    }
    if (lc < NL) {
        k_mg_coarse<T><<<N, MG_COARSE_THREADS, 0, s>>>(b.dcases, tab, lc, NL, nuc, ncoarse);
        count_launch();
    } else {
        for (int it = 0; it < ncoarse; ++it) {
            launch_smooth<T>(b, tab, NL - 1, 0, it == 0, s);
            launch_smooth<T>(b, tab, NL - 1, 1, 0, s);
        }
        count_launch(2 * ncoarse);
    }
    for (int l = ldown - 1; l >= 0; --l) {
        const int nu = (l == 0) ? nu0 : nuc;
        if (fused) {
            // black then red; the prolongation writes the buffer the first
            // sweep reads, chosen so that the last sweep writes z
            k_mg_prolong<T><<<gP, b.cblock(), 0, s>>>(b.dcases, tab, N, l, nu & 1);
            for (int it = 0; it < nu; ++it) {
                const int dst = (nu - 1 - it) & 1;
                k_mg_sweep<T><<<gW, b.cblock(), SW_SMEM, s>>>(b.dcases, tab, N, l, 1, 0, 1 - dst, dst);
            }
            count_launch(nu + 1);
            continue;
        }
        k_mg_prolong<T><<<gP, b.cblock(), 0, s>>>(b.dcases, tab, N, l, 0);
        for (int it = 0; it < nu; ++it) {
            launch_smooth<T>(b, tab, l, 1, 0, s);
            launch_smooth<T>(b, tab, l, 0, 0, s);
        }
        count_launch(2 * nu + 1);
    }
}

// profiling: one red half-sweep on level 0 over table `tab`
template <typename T> int launch_mg_smooth0(const Batch<T> &b, const int *tab, int grid, cudaStream_t s)
{
    (void)grid;
    if (b.nlev < 2) return -1;
    launch_smooth<T>(b, tab, 0, 0, 0, s);
    count_launch();
    return 0;
}
template <> int launch_mg_smooth0<double>(const Batch<double> &, const int *, int, cudaStream_t) { return -1; }

// profiling: one whole one-pass sweep on level 0 (z -> z2) over table `tab`
template <typename T> int launch_mg_sweep0(const Batch<T> &b, const int *tab, cudaStream_t s)
{
    if (b.nlev < 2) return -1;
    const int gW = sweep_grid<T>(b);
    k_mg_sweep<T><<<gW, b.cblock(), SW_SMEM, s>>>(b.dcases, tab, b.ncases, 0, 0, 0, 0, 1);
    count_launch();
    return 0;
}
template <> int launch_mg_sweep0<double>(const Batch<double> &, const int *, cudaStream_t) { return -1; }

// profiling and tuning: one V-cycle over table `tab` (mixed form with the
// multigrid passes only)
template <typename T> int launch_mg_vcycle_prof(const Batch<T> &b, const int *tab, cudaStream_t s)
{
    if (b.nlev < 2) return -1;
    launch_mg_vcycle<T>(b, tab, 0, s);
    return 0;
}
template <> int launch_mg_vcycle_prof<double>(const Batch<double> &, const int *, cudaStream_t) { return -1; }

template int launch_mg_vcycle_prof<float>(const Batch<float> &, const int *, cudaStream_t);
template void launch_mg_coarsen<float>(const Batch<float> &, cudaStream_t);
template int launch_mg_smooth0<float>(const Batch<float> &, const int *, int, cudaStream_t);
template int launch_mg_sweep0<float>(const Batch<float> &, const int *, cudaStream_t);
template void launch_mg_vcycle<float>(const Batch<float> &, const int *, int, cudaStream_t);

}  // namespace suli
