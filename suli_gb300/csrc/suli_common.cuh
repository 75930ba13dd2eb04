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

#include <cuda_runtime.h>
#include <stdint.h>

namespace suli {

constexpr int TX = 32;   // tile = thread block, one cell per thread
constexpr int TY = 4;
constexpr int TZ = 2;
constexpr int NTHREADS = TX * TY * TZ;
constexpr int NSLOT = 8; // reduction slots per block

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
    S_NSCAL
};

struct Geo {
    int nx, ny, nz;
    int pad;
    long long sx, sxy, total;
    __host__ __device__ __forceinline__ long long at(int i, int j, int k) const
    {
        return (long long)i + sx * (long long)j + sxy * (long long)k;
    }
};

template <typename T>
struct CaseDev {
    Geo g;
    // tiles of this case in the launch grid
    int tile_begin, ntiles, ntx, nty, ntz;
    // discretisation / physics (double in both forms)
    double dx, dy, dz, dx1, dt1, deltai;
    double alpha1, rho_f1, mu_f1, rho_f2, mu_f2, gx, gz;
    double cles;         // (dx*dy*dz)^(2/3) * csmag * csmag
    double pi;
    double uinicial, iturb;
    unsigned long long seed;
    int ccx0, ccxf, ccy0, ccyf, ccz0, cczf;
    int t_tempo, m_turb, mms_t, ibm_t, obst_t;
    int reinit_max, cg_max, cg_tol_mode;
    double cg_tol;
    // fields (reference module arrays)
    T *u, *v, *w, *prd1, *prd;
    T *ls, *lsb, *lsc, *funcs, *hs, *rho, *ls_mu, *mu, *mut, *xmu, *ymu, *zmu;
    T *Fu, *Fv, *Fw, *u0, *v0, *w0, *fu0, *fv0, *fw0, *fu1, *fv1, *fw1;
    T *div, *tf_u, *tf_v, *tf_w;
    T *obs_lsx, *obs_lsy, *obs_lsz, *obs_lss;
    int *id_ibmx, *id_ibmy, *id_ibmz, *id_ibm;
    T *bxx0, *bxx1, *blx1;      // inflow planes, indexed at(0, j, k)
    // CG work arrays
    T *spi, *spj, *spk, *dpr, *e, *r, *p, *mp, *qpr;
    double *e64, *r64;          // mixed form: FP64 refinement vectors
    // reductions
    double *sc;                 // S_NSCAL scalars of this case
    double *partials;           // NSLOT * total_tiles (global base, slot-major)
    unsigned int *counter;      // one per case
    int total_tiles;            // of the whole launch (slot stride)
};

// ---- tile decode ---------------------------------------------------------
template <typename T>
__device__ __forceinline__ int find_case(const CaseDev<T> *cs, int ncases)
{
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
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
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

// Publish NS per-block partial values; returns true in every thread of the
// last block of the case to arrive, after which `tot` holds the case totals
// (sums for slots with maxmask bit clear, maxima otherwise), reduced in a
// fixed order so results do not depend on block scheduling.
template <typename T, int NS>
__device__ bool last_block_reduce(const CaseDev<T> &c, const double (&vals)[NS], double (&tot)[NS],
                                  unsigned maxmask = 0u)
{
    __shared__ double sh[32];
    __shared__ bool amlast;
    double bv[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s)
        bv[s] = ((maxmask >> s) & 1u) ? block_max(vals[s], sh) : block_sum(vals[s], sh);
    int t = tid_lin();
    if (t == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) c.partials[(long long)s * c.total_tiles + blockIdx.x] = bv[s];
        __threadfence();
        unsigned prev = atomicAdd(c.counter, 1u);
        amlast = (prev == (unsigned)(c.ntiles - 1));
    }
    __syncthreads();
    if (!amlast) return false;
    __threadfence();
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        bool ismax = (maxmask >> s) & 1u;
        double a = ismax ? 0.0 : 0.0;
        const double *src = c.partials + (long long)s * c.total_tiles + c.tile_begin;
        for (int q = t; q < c.ntiles; q += NTHREADS) {
            double x = __ldcg(src + q);
            a = ismax ? fmax(a, x) : a + x;
        }
        tot[s] = ismax ? block_max(a, sh) : block_sum(a, sh);
    }
    if (t == 0) *c.counter = 0u;
    return true;
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
