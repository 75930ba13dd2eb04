// suli_common.cuh -- shared device-side definitions of the SuLi GB300 kernels.
//
// Every kernel is batched: it takes a table of cases (one for a single run,
// hundreds for an ensemble) and a 1-D grid of tiles; block b finds its case
// by a binary search over the per-case tile offsets.  All arrays of a case
// share one padded box layout:
//
//   idx(i,j,k) = i + sx*j + sxy*k,   i in [0, nx+2], j in [0, ny+2], k in [0, nz+2]
//
// which holds every staggered array of the reference with its ghost layer
// (u (0:nx+2,0:ny+1,0:nz+1), v, w, prd1, and the cell/face arrays that start
// at 1), i (x) unit-stride as in the Fortran column-major originals.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace suli {

constexpr int TX = 32;   // tile = thread block, one cell per thread
constexpr int TY = 4;
constexpr int TZ = 2;
constexpr int NTHREADS = TX * TY * TZ;
constexpr int NSLOT = 8; // reduction slots per block
// work unit of the persistent kernels on the case grid: a column of
// COL_X x COL_Y cells in x, y (one per thread of a 32 x 8 block) and COL_Z
// planes, which each thread walks in groups of COL_G planes
constexpr int COL_X = 32, COL_Y = 8, COL_Z = 8;
constexpr int COL_G = 4;   // planes a thread loads before it computes (one group)
__host__ __device__ __forceinline__ int col_units(int nx, int ny, int nz)
{
    return ((nx + COL_X - 1) / COL_X) * ((ny + COL_Y - 1) / COL_Y) * ((nz + COL_Z - 1) / COL_Z);
}

// per-case device scalars (double), indices into CaseDev::sc
enum Scal {
    S_DT = 0,      // stage dt (a_dt(tt))
    S_DTADV,       // dt used by the level-set advection
    S_RR,          // CG r.r (alfamupr)
    S_RR0,
    S_ALPHA,
    S_BETA,
    S_THR,         // CG stop threshold on r.r
    S_CGACTIVE,    // 1 while the CG of this case iterates
    S_CGITER,
    S_RINACTIVE,   // 1 while reinitialisation iterates
    S_RINITER,
    S_RINREPLAY,   // >= 0: replay this many reinit iterations
    S_CGREPLAY,    // >= 0: replay this many CG iterations
    S_VOLINI,
    S_VOLINS,
    S_VOLACTIVE,
    S_MAXDIV,
    S_BANDSUM,
    S_BANDCNT,
    S_CGMAX,
    S_ERR0, S_ERR1, S_ERR2, S_ERR3,     // MMS errors
    S_RRTRUE,      // mixed form: FP64 true residual r.r
    S_OUTER,       // mixed form: FP64 residual passes (negative once converged)
    S_UPDATE,      // mixed form: 1 while a reliable update is pending
    S_RRREF,       // mixed form: FP32 r.r at the last update
    S_RRPREV,      // mixed form: r.r before the pending update
    S_RZ,          // mixed form, multigrid-preconditioned passes: r.z
    S_P64OK,       // mixed form: e64 holds the FP64 pressure of the last solve
    S_PASS0,       // mixed form: CG iteration count at the start of the pass
    S_IDT,         // 1 / dt of the stage (host-set beside S_DT)
    S_STALL,       // mixed form: consecutive passes that did not halve the best FP64 r.r
    S_RRBEST,      // mixed form: the lowest FP64 r.r of the solve so far
    S_STALLED,     // mixed form: 1 when the refinement ended on stagnation
    S_TMAERR,      // 1 when a bounded wait for a TMA copy gave up (SULI_DEVICE_TIMEOUT)
    // whole-step graph: per stage the solve's iterations and FP64 passes,
    // stagnation in any stage; in case 0 the device loops' trip counters
    S_STIT0, S_STIT1, S_STIT2,
    S_STOUT0, S_STOUT1, S_STOUT2,
    S_STSTALL,
    S_TRIP_VOL, S_TRIP_OUT0, S_TRIP_OUT1, S_TRIP_OUT2, S_TRIP_IN0, S_TRIP_IN1, S_TRIP_IN2,
    // in case 0: the step's host values the step graph's launches read (the
    // step number, the time, the inflow's random-number call count at the
    // start of the step); contiguous, written by one copy per step
    S_ITSTEP, S_TIME, S_RNGBASE,
    S_NSCAL
};

// 1/x in FP64 without a division, for the mixed form's FP64 kernels (an
// FP64 divide is a long instruction sequence on GB300's FP64 units): an FP32
// reciprocal as seed and two Newton-Raphson steps r <- r + r (1 - x r), each
// doubling the correct bits (24 -> 48 -> FP64, within a few ulps).  x must
// be a normal number inside the FP32 range (densities, face conductances).
__device__ __forceinline__ double rcp_nr64(double x)
{
    double r = (double)__frcp_rn((float)x);
    r = fma(r, fma(-x, r, 1.0), r);
    r = fma(r, fma(-x, r, 1.0), r);
    return r;
}

struct Geo {
    int nx, ny, nz;
    int pad;
    long long sx, sxy, total;
    __host__ __device__ __forceinline__ long long at(int i, int j, int k) const
    {
        return (long long)i + sx * (long long)j + sxy * (long long)k;
    }
};

// One multigrid level of a case (mixed form).  Level 0 is the case's own grid
// and box; coarser levels halve each dimension (n -> (n+1)/2, cell I owning
// fine cells 2I-1 and 2I) in a box laid out like the case's (rows of a
// multiple of 8 elements, 32-byte aligned, so the one-pass sweep's 16-byte
// copies apply on every level).
// cx(i,j,k) is the conductance of the face between cells i-1 and i (zero on
// a Neumann wall), dg the sum of a cell's six face conductances.
constexpr int MG_MAXL = 12;
template <typename T>
struct MgLev {
    Geo g;
    int ntx, nty, ntz, ntiles;
    int ncols;    // column units of the level (col_units): its active-table units
    T *cx, *cy, *cz, *dg, *z, *f;
    T *dgi;    // 1 / dg (0 where dg = 0): the smoothers multiply instead of divide
    T *z2;     // the second buffer of the one-pass sweeps
};

template <typename T>
struct CaseDev {
    Geo g;
    // tiles of this case in the launch grid
    int tile_begin, ntiles, ntx, nty, ntz;
    const int *tile_case;       // case of each tile of the launch grid (the same table in every case)
    // column units of the case grid (the unit of the persistent CG kernels
    // and of their reductions), see col_units
    int chunk_begin, nchunks;
    // first unit of this case in the launch grid of the TMA-staged convdiff,
    // and its first boundary-shell position in the shell kernel's grid
    int cd_begin[3];            // per unit height of the tuner's choice (8, 16, 32 planes)
    long long cd_shell_begin;
    // discretisation / physics (double in both forms)
    double dx, dy, dz, dx1, dt1, deltai;
    double idx, idy, idz;       // 1/dx, 1/dy, 1/dz (mixed-form kernels multiply)
    // FP32 roundings of idx, idy, idz for the FP32 kernels (a conversion per
    // thread runs on GB300's FP64 pipe)
    float fidx, fidy, fidz;
    double alpha1, rho_f1, mu_f1, rho_f2, mu_f2, gx, gz;
    double sigma;               // surface tension coefficient (t_tens = 1)
    double cles;         // (dx*dy*dz)^(2/3) * csmag * csmag
    double pi;
    double uinicial, iturb;
    double cmu, cdes, lcar, delta;   // k equation (m_turb >= 2); delta = max(dx, dy, dz)
    unsigned long long seed;
    int ccx0, ccxf, ccy0, ccyf, ccz0, cczf;
    int t_tempo, m_turb, mms_t, ibm_t, obst_t, t_tens;
    int t_press, ipa;           // ipa: t_press = 2 and the step projects (exp_press / IPA graddin)
    int esp_type;               // sponge layer (0 none)
    int wave_t;                 // inflow waves (0 none, 1/2 Stokes I/II, 5 Stokes V)
    int outflow_flux;           // 1: contorno(2) balances the free-outflow faces' flux to the inflow's
    // SuLi-ICdz's variable z spacing (dz_t = 1, else all null): dz(k) and
    // dzz(k) for k = 0..nz+1 with their reciprocals, and the WENO z
    // spacing dz11(m), m = -2..nz+3 (dz11 points at m = 0)
    const double *dzk, *dzzk, *idzk, *idzzk, *dz11;
    double a_w, f_w, n_w, h0_f, aeta[5], avel[5];   // waves_coef's results
    int reinit_max, cg_max, cg_tol_mode;
    double cg_tol;
    // fields (reference module arrays)
    T *u, *v, *w, *prd1, *prd;
    T *ls, *lsb, *lsc, *funcs, *hs, *rho, *ls_mu, *mu, *mut, *xmu, *ymu, *zmu;
    T *Fu, *Fv, *Fw, *u0, *v0, *w0, *fu0, *fv0, *fw0, *fu1, *fv1, *fw1;
    T *div, *tf_u, *tf_v, *tf_w;
    T *obs_lsx, *obs_lsy, *obs_lsz, *obs_lss;
    T *obs_ls;                  // obstacle level set at the cell corners (field output only)
    T *hsx, *hsy, *hsz, *kurv;  // surface tension (t_tens = 1): weights, curvature
    T *nlx, *nly, *nlz;         // surface tension: the interface normal (curvature input)
    // k equation (m_turb >= 2, else null): ka with its ghosts, nut, the strain
    // sum p1 + p2 + p3 of visco, and the sub-stage buffers of tempo_esc (e0,
    // fe0, fe1) and of the stage's right-hand side
    T *ka, *nut, *sij, *ka0, *fk0, *fk1, *fka;
    // IPA (t_press = 2, else null): accumulated pressure and the explicit force
    T *prd0, *px, *py, *pz;
    // sponge layer (esp_type > 0, else null): epis_z on the w faces
    T *epis;
    int *id_ibmx, *id_ibmy, *id_ibmz, *id_ibm;
    T *bxx0, *bxx1, *blx1, *bxz0;   // inflow planes, element (j, k) at j + (ny + 3) k
    // CG work arrays
    T *spi, *spj, *spk, *dpr, *e, *r, *p, *mp, *qpr;
    double *e64, *r64;          // mixed form: FP64 refined solution (after the solve: the FP64
                                // pressure); 1/sqrt(D) of the cached operator
    // mixed form: FP64 pressure operator for the refinement residual (density
    // from the FP32 level set in FP64, scaled face coefficients, diagonal, rhs)
    double *rho64, *spi64, *spj64, *spk64, *dpr64, *qpr64;
    // mixed form: FP64 masters of the velocity and of its RK stage copy.  The
    // FP32 u, v, w (and u0 ...) are what every stencil reads; the masters are
    // what tempo and posdin accumulate into (an FP32 predictor carries the
    // gravity increment, and rounding it leaves noise that the variable-
    // density projection moves into the light phase)
    double *u64, *v64, *w64, *u064, *v064, *w064;
    // mixed form: the projection's FP64 unit face factors 1 / (h rho_face) of
    // the cached pressure operator (written by k_cg_op1m, read by posdin)
    double *pfx64, *pfy64, *pfz64;
    // mixed form: FP64 masters of the level set and its two RK stage buffers
    // (WENO reads the FP32 copies; the stage combinations of advection,
    // reinitialisation and the volume correction accumulate in FP64)
    double *ls64, *lsb64, *lsc64;
    // multigrid hierarchy of the mixed form's preconditioner (nlev = 0: none)
    int nlev;
    MgLev<T> mg[MG_MAXL];
    // reductions
    double *sc;                 // S_NSCAL scalars of this case
    double *partials;           // NSLOT * pstride (global base, slot-major)
    int pstride;                // slot stride of partials: max(tiles, 8 x column units) of the batch
    unsigned int *counter;      // one per case
    int total_tiles;            // of the whole launch (slot stride)
};

// ---- tile decode ---------------------------------------------------------
// a per-case constant in the kernel's precision: the stored FP32 rounding
// in FP32, the FP64 value in FP64
template <typename T> __device__ __forceinline__ T cval(double d, float f)
{
    if constexpr (sizeof(T) == 4) return f;
    else return d;
}

template <typename T>
__device__ __forceinline__ int find_case(const CaseDev<T> *cs, int ncases)
{
    if (const int *tc = cs[0].tile_case) return tc[blockIdx.x];
    int b = blockIdx.x;
    int lo = 0, hi = ncases - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (cs[mid].tile_begin <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <typename T>
__device__ __forceinline__ void tile_ijk(const CaseDev<T> &c, int &i, int &j, int &k)
{
    int t = blockIdx.x - c.tile_begin;
    int ti = t % c.ntx;
    int r = t / c.ntx;
    int tj = r % c.nty;
    int tk = r / c.nty;
    i = 1 + ti * TX + (int)threadIdx.x;
    j = 1 + tj * TY + (int)threadIdx.y;
    k = 1 + tk * TZ + (int)threadIdx.z;
}

__device__ __forceinline__ int tid_lin() { return threadIdx.x + TX * (threadIdx.y + TY * threadIdx.z); }

// ---- deterministic block reduction ----------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
// maximum of non-negative values (+0.0, never -0.0; +inf for a NaN): their
// bit patterns order as unsigned integers, so the maximum runs on the integer
// units instead of GB300's FP64 pipe, exactly
__device__ __forceinline__ double warp_max(double v)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_down_sync(0xffffffffu, b, o));
    return __longlong_as_double((long long)b);
}

// sum over the block in a fixed order; result valid in thread 0
__device__ __forceinline__ double block_sum(double v, double *sh)
{
    int t = tid_lin();
    v = warp_sum(v);
    if ((t & 31) == 0) sh[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        v = (t < NTHREADS / 32) ? sh[t] : 0.0;
        v = warp_sum(v);
    }
    __syncthreads();
    return v;
}
__device__ __forceinline__ double block_max(double v, double *sh)
{
    int t = tid_lin();
    v = warp_max(v);
    if ((t & 31) == 0) sh[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        v = (t < NTHREADS / 32) ? sh[t] : 0.0;
        v = warp_max(v);
    }
    __syncthreads();
    return v;
}

// unit_reduce: publish NS per-unit partial values of unit `gunit` (global
// unit id); returns true in every thread of the block that completes the
// case's last unit, after which `tot` holds the case totals (sums for slots
// with maxmask bit clear, maxima of non-negative values otherwise), reduced
// in unit order so results do not depend on block scheduling.
// unit_publish is its second half, from the block's values in thread 0 (bv).
template <typename T, int NS>
__device__ bool unit_publish(const CaseDev<T> &c, int gunit, int ubegin, int nunits, const double (&bv)[NS],
                             double (&tot)[NS], unsigned maxmask, double *sh)
{
    __shared__ bool amlast;
    int t = tid_lin();
    if (t == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) c.partials[(long long)s * c.pstride + gunit] = bv[s];
        __threadfence();
        unsigned prev = atomicAdd(c.counter, 1u);
        amlast = (prev == (unsigned)(nunits - 1));
    }
    __syncthreads();
    if (!amlast) return false;
    __threadfence();
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        bool ismax = (maxmask >> s) & 1u;
        double a = ismax ? 0.0 : 0.0;
        const double *src = c.partials + (long long)s * c.pstride + ubegin;
        for (int q = t; q < nunits; q += NTHREADS) {
            double x = __ldcg(src + q);
            a = ismax ? fmax(a, x) : a + x;
        }
        tot[s] = ismax ? block_max(a, sh) : block_sum(a, sh);
    }
    if (t == 0) *c.counter = 0u;
    return true;
}
template <typename T, int NS>
__device__ bool unit_reduce(const CaseDev<T> &c, int gunit, int ubegin, int nunits, const double (&vals)[NS],
                            double (&tot)[NS], unsigned maxmask = 0u)
{
    __shared__ double sh[32];
    double bv[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s)
        bv[s] = ((maxmask >> s) & 1u) ? block_max(vals[s], sh) : block_sum(vals[s], sh);
    return unit_publish<T, NS>(c, gunit, ubegin, nunits, bv, tot, maxmask, sh);
}

// unit_reduce of sums of FP32 thread values (mixed form): each warp sums its
// 32 values in FP32 in a fixed shuffle order (a relative 1e-6 at worst, on
// quantities that feed stopping tests and diagnostics), lane 0 widens the
// warp's sum, times wscale[s] (a per-warp factor, e.g. a cell volume that
// is uniform along a warp's x-row), and thread 0 adds the block's warps in
// FP64: one FP64 operation per warp instead of a five-level FP64 shuffle
// tree per thread on GB300's FP64 pipe
template <typename T, int NS>
__device__ bool unit_reduce_f32(const CaseDev<T> &c, int gunit, int ubegin, int nunits, const float (&vals)[NS],
                                const double (&wscale)[NS], double (&tot)[NS])
{
    __shared__ double sh[NS * (NTHREADS / 32)];
    const int t = tid_lin();
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        float v = vals[s];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((t & 31) == 0) sh[s * (NTHREADS / 32) + (t >> 5)] = (double)v * wscale[s];
    }
    __syncthreads();
    double bv[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        double a = 0.0;
        if (t == 0)
            for (int w = 0; w < NTHREADS / 32; ++w) a += sh[s * (NTHREADS / 32) + w];
        bv[s] = a;
    }
    __shared__ double sh2[32];
    return unit_publish<T, NS>(c, gunit, ubegin, nunits, bv, tot, 0u, sh2);
}

// one tile per block (the launch grid is the tile grid)
template <typename T, int NS>
__device__ __forceinline__ bool last_block_reduce(const CaseDev<T> &c, const double (&vals)[NS], double (&tot)[NS],
                                                  unsigned maxmask = 0u)
{
    return unit_reduce<T, NS>(c, (int)blockIdx.x, c.tile_begin, c.ntiles, vals, tot, maxmask);
}
template <typename T, int NS>
__device__ __forceinline__ bool last_block_reduce_f32(const CaseDev<T> &c, const float (&vals)[NS],
                                                      const double (&wscale)[NS], double (&tot)[NS])
{
    return unit_reduce_f32<T, NS>(c, (int)blockIdx.x, c.tile_begin, c.ntiles, vals, wscale, tot);
}


// ---- active-case tables (persistent CG iteration) ---------------------------
// A table lists the cases whose CG still iterates and, per grid level s, the
// prefix of their work-unit counts, so a fixed grid can walk exactly the
// active units of a level.  Level 0 is the case grid, level s > 0 multigrid
// level s; the unit is a column unit of the level (column_of):
//   tab[0] = n, tab[1 .. 1+n) = case ids,
//   level s at B = 1 + N + s (N + 2): tab[B] = units, tab[B+1 .. B+1+n] = prefix
// (N = cases in the batch, NL = levels in the table).
__host__ __device__ __forceinline__ int act_stride(int ncases, int nl) { return 1 + ncases + nl * (ncases + 2); }
__host__ __device__ __forceinline__ int act_level(int ncases, int s) { return 1 + ncases + s * (ncases + 2); }

// this thread's offset inside a TX x TY x TZ tile, from its linear id (so a
// kernel may run with 32 x 4 x 2 or 32 x 8 x 1 blocks)
__device__ __forceinline__ int tile_ox() { return tid_lin() & (TX - 1); }
__device__ __forceinline__ int tile_oy() { return (tid_lin() / TX) % TY; }
__device__ __forceinline__ int tile_oz() { return tid_lin() / (TX * TY); }

// tile `lt` of a grid with ntx x nty tiles -> the cell of this thread
__device__ __forceinline__ void tile_cell(int ntx, int nty, int lt, int &i, int &j, int &k)
{
    int ti = lt % ntx;
    int r = lt / ntx;
    int tj = r % nty;
    int tk = r / nty;
    i = 1 + ti * TX + tile_ox();
    j = 1 + tj * TY + tile_oy();
    k = 1 + tk * TZ + tile_oz();
}

// column unit u of a grid (see COL_X): this thread's (i, j), clamped into the
// grid (v = false outside it), and the planes k0..k1 the column covers.
// Needs 256 threads per block.
struct Column {
    int i, j, k0, k1;
    bool v;
};
__device__ __forceinline__ Column column_of(const Geo &g, int u)
{
    const int ux = (g.nx + COL_X - 1) / COL_X, uy = (g.ny + COL_Y - 1) / COL_Y;
    const int a = u % ux, r = u / ux, b = r % uy, cz = r / uy;
    const int t = tid_lin();
    const int i = 1 + a * COL_X + (t & (COL_X - 1)), j = 1 + b * COL_Y + t / COL_X;
    Column c;
    c.v = i <= g.nx && j <= g.ny;
    c.i = min(i, g.nx);
    c.j = min(j, g.ny);
    c.k0 = 1 + cz * COL_Z;
    c.k1 = min(g.nz, c.k0 + COL_Z - 1);
    return c;
}

template <typename T>
__device__ __forceinline__ void tile_ijk_of(const CaseDev<T> &c, int lt, int &i, int &j, int &k)
{
    tile_cell(c.ntx, c.nty, lt, i, j, k);
}

// The cells of this thread in U consecutive tiles of a unit, so a kernel can
// issue the loads of several cells before it uses any (memory parallelism):
// the walk decodes the unit's first tile once and then steps x-tile, y-tile,
// z-tile without divisions.  Cells outside the grid (tile padding, tiles past
// the unit) come back clamped to the nearest interior cell with v = false, so
// loads at them stay in bounds and can be issued without a branch.
struct TileWalk {
    int ti, tj, tk, ntx, nty;
    __device__ __forceinline__ TileWalk(int t0, int ntx_, int nty_) : ntx(ntx_), nty(nty_)
    {
        ti = t0 % ntx;
        int r = t0 / ntx;
        tj = r % nty;
        tk = r / nty;
    }
    template <int U>
    __device__ __forceinline__ void next(int lt, int t1, const Geo &g, long long (&q)[U], int (&ci)[U],
                                         int (&cj)[U], int (&ck)[U], bool (&v)[U])
    {
#pragma unroll
        for (int a = 0; a < U; ++a) {
            const int i = 1 + ti * TX + tile_ox();
            const int j = 1 + tj * TY + tile_oy();
            const int k = 1 + tk * TZ + tile_oz();
            v[a] = (lt + a < t1) && i <= g.nx && j <= g.ny && k <= g.nz;
            ci[a] = min(i, g.nx);
            cj[a] = min(j, g.ny);
            ck[a] = min(k, g.nz);
            q[a] = g.at(ci[a], cj[a], ck[a]);
            if (++ti == ntx) {
                ti = 0;
                if (++tj == nty) { tj = 0; ++tk; }
            }
        }
    }
};
constexpr int UW = 2;   // cells per thread per step of the walk



// Block b of the grid takes the contiguous range of active units of level s,
// [U b / G, U (b+1) / G), and calls f(case id, local unit) for each, in
// order.  Every thread of the block makes the same calls.
template <typename F>
__device__ __forceinline__ void for_active_units(const int *__restrict__ tab, int N, int s, F f)
{
    const int n = tab[0];
    const int *ids = tab + 1;
    const int *lv = tab + act_level(N, s);
    const int tiles = lv[0];
    const int *off = lv + 1;
    const int lo = (int)((long long)tiles * blockIdx.x / gridDim.x);
    const int hi = (int)((long long)tiles * (blockIdx.x + 1) / gridDim.x);
    if (lo >= hi) return;
    int a0 = 0, a1 = n - 1;        // last slot with off <= lo
    while (a0 < a1) {
        int mid = (a0 + a1 + 1) >> 1;
        if (off[mid] <= lo) a0 = mid; else a1 = mid - 1;
    }
    int a = a0;
    int end = off[a + 1];
    for (int t = lo; t < hi; ++t) {
        while (t >= end) { ++a; end = off[a + 1]; }
        f(ids[a], t - off[a]);
    }
}

// The active units of level s dealt round-robin: block b takes units b,
// b + G, b + 2G, ... (G blocks), so neighbouring units run at the same time
// on different blocks (their shared halo is read from DRAM once and hits in
// L2 for the other).  Every thread of the block makes the same calls.
template <typename F>
__device__ __forceinline__ void for_active_units_rr(const int *__restrict__ tab, int N, int s, F f)
{
    const int n = tab[0];
    const int *ids = tab + 1;
    const int *lv = tab + act_level(N, s);
    const int units = lv[0];
    const int *off = lv + 1;
    int a = 0;
    for (int t = blockIdx.x; t < units; t += gridDim.x) {
        int a1 = n - 1;              // last slot with off <= t (at or after the previous one)
        while (a < a1) {
            const int mid = (a + a1 + 1) >> 1;
            if (off[mid] <= t) a = mid; else a1 = mid - 1;
        }
        f(ids[a], t - off[a]);
    }
}

// As for_active_units, for kernels that reduce per unit: unit(id, u) runs
// for each unit; seg(id, n) runs once after the block's last unit of a case
// in its range (n = units it did for that case), so the completion fence
// and atomic of a reduction are paid per segment, not per unit.
template <typename F, typename G>
__device__ __forceinline__ void for_active_units_seg(const int *__restrict__ tab, int N, int s, F unit, G seg)
{
    const int n = tab[0];
    const int *ids = tab + 1;
    const int *lv = tab + act_level(N, s);
    const int tiles = lv[0];
    const int *off = lv + 1;
    const int lo = (int)((long long)tiles * blockIdx.x / gridDim.x);
    const int hi = (int)((long long)tiles * (blockIdx.x + 1) / gridDim.x);
    if (lo >= hi) return;
    int a0 = 0, a1 = n - 1;
    while (a0 < a1) {
        int mid = (a0 + a1 + 1) >> 1;
        if (off[mid] <= lo) a0 = mid; else a1 = mid - 1;
    }
    int a = a0;
    int end = off[a + 1];
    int cnt = 0;
    for (int t = lo; t < hi; ++t) {
        while (t >= end) {
            if (cnt > 0) seg(ids[a], cnt);
            cnt = 0;
            ++a;
            end = off[a + 1];
        }
        unit(ids[a], t - off[a]);
        ++cnt;
    }
    if (cnt > 0) seg(ids[a], cnt);
}

// the partials of one column unit: one per warp (a shuffle sum, no block
// barrier), at (unit, warp) of the case; no fence, no counter (seg_reduce)
constexpr int UNIT_WARPS = NTHREADS / 32;
template <typename T, int NS>
__device__ __forceinline__ void unit_partial(const CaseDev<T> &c, int u, const double (&vals)[NS])
{
    const int t = tid_lin();
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const double v = warp_sum(vals[s]);
        if ((t & 31) == 0)
            c.partials[(long long)s * c.pstride + (long long)(c.chunk_begin + u) * UNIT_WARPS + (t >> 5)] = v;
    }
}

// one partial of a unit from a thread value in the storage type: in FP32 the
// warp sums in FP32 (a fixed shuffle order) and lane 0 widens the warp's sum
// to the FP64 partial, so the FP64 pipe (a small fraction of GB300's FP32
// rate) sees one conversion per warp; in FP64 as unit_partial
template <typename T>
__device__ __forceinline__ void unit_partial1(const CaseDev<T> &c, int u, T v)
{
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        const int t = tid_lin();
        if ((t & 31) == 0) c.partials[(long long)(c.chunk_begin + u) * UNIT_WARPS + (t >> 5)] = (double)v;
    } else {
        const double vals[1] = {(double)v};
        unit_partial<T, 1>(c, u, vals);
    }
}

// end of a segment of `cnt` units of case c: returns true in every thread of
// the block that completes the case's last unit, with the totals over the
// case's warp partials (summed in (unit, warp) order) in tot
template <typename T, int NS>
__device__ bool seg_reduce(const CaseDev<T> &c, int cnt, double (&tot)[NS])
{
    __shared__ double sh[32];
    __shared__ bool amlast;
    const int t = tid_lin();
    if ((t & 31) == 0) __threadfence();   // this warp's partials of the segment
    __syncthreads();
    if (t == 0) {
        const unsigned prev = atomicAdd(c.counter, (unsigned)cnt);
        amlast = (prev + (unsigned)cnt == (unsigned)c.nchunks);
    }
    __syncthreads();
    if (!amlast) return false;
    __threadfence();
    const int np = c.nchunks * UNIT_WARPS;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        double a = 0.0;
        const double *src = c.partials + (long long)s * c.pstride + (long long)c.chunk_begin * UNIT_WARPS;
        for (int q = t; q < np; q += NTHREADS) a += __ldcg(src + q);
        tot[s] = block_sum(a, sh);
    }
    if (t == 0) *c.counter = 0u;
    return true;
}

// exclusive prefix sum over the block (NTHREADS threads, linear id order);
// *total gets the sum.  Contains __syncthreads: call from every thread.
__device__ __forceinline__ int block_exscan(int v, int *total)
{
    __shared__ int wsum[NTHREADS / 32];
    const int t = tid_lin(), lane = t & 31, w = t >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = (lane < NTHREADS / 32) ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < NTHREADS / 32) wsum[lane] = s;   // inclusive warp prefix
    }
    __syncthreads();
    const int before = (w > 0) ? wsum[w - 1] : 0;
    *total = wsum[NTHREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// Build table `out` (NL levels) from the cases listed in `in` (or all N
// cases when in is null) whose S_CGACTIVE flag is set (every case when
// `all`), keeping their order.  One block; every thread calls it.
template <typename T>
__device__ void build_active_table(const CaseDev<T> *__restrict__ cs, int N, int NL, const int *in, int *out,
                                   bool all = false)
{
    const int nin = in ? in[0] : N;
    const int t = tid_lin();
    const int per = (nin + NTHREADS - 1) / NTHREADS;
    const int a0 = min(nin, t * per), a1 = min(nin, a0 + per);
    // the active flags of this thread's cases, read once (bit a - a0; a
    // thread with more than 64 cases re-reads them per level)
    const bool cached = per <= 64;
    unsigned long long am = 0ull;
    int cnt = 0;
    for (int a = a0; a < a1; ++a) {
        const int id = in ? in[1 + a] : a;
        if (all || __ldcg(&cs[id].sc[S_CGACTIVE]) != 0.0) {
            if (cached) am |= 1ull << (a - a0);
            ++cnt;
        }
    }
    auto active = [&](int a, int id) {
        return cached ? ((am >> (a - a0)) & 1ull) != 0ull : (all || __ldcg(&cs[id].sc[S_CGACTIVE]) != 0.0);
    };
    int ncnt;
    const int pos0 = block_exscan(cnt, &ncnt);
    // units of level s of case id
    auto units = [&](int id, int s) { return s == 0 ? cs[id].nchunks : cs[id].mg[s].ncols; };
    for (int s = 0; s < NL; ++s) {
        int til = 0;
        for (int a = a0; a < a1; ++a) {
            const int id = in ? in[1 + a] : a;
            if (active(a, id)) til += units(id, s);
        }
        int ntil;
        int tpos = block_exscan(til, &ntil);
        int *lv = out + act_level(N, s);
        int pos = pos0;
        for (int a = a0; a < a1; ++a) {
            const int id = in ? in[1 + a] : a;
            if (active(a, id)) {
                if (s == 0) out[1 + pos] = id;
                lv[1 + pos] = tpos;
                ++pos;
                tpos += units(id, s);
            }
        }
        if (t == 0) {
            lv[0] = ntil;
            lv[1 + ncnt] = ntil;
        }
    }
    if (t == 0) out[0] = ncnt;
}

// counter-based hash RNG in [0,1): the same function runs in the oracle
__host__ __device__ __forceinline__ double rng_uniform(unsigned long long seed, unsigned long long ctr)
{
    unsigned long long z = seed + 0x9E3779B97F4A7C15ULL * (ctr + 1ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace suli
