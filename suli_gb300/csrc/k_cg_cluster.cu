// k_cg_cluster.cu -- the CG iteration loop of graddin (9_grad.f90:398-587)
// for batches of small cases, one thread-block cluster per case.
//
// A cluster of CL CTAs (8, or 16 where the part allows it) owns one case: CTA
// `rank` sweeps the z-slab k in [k0, k1) of the case.  The whole loop runs in
// one launch:
//   phase A   mp = A p over the slab, block partial of p.mp
//   reduce    each CTA publishes its partial in shared memory, one
//             barrier.cluster, then every CTA sums the CL partials through
//             distributed shared memory in rank order -- identical totals in
//             all CTAs, so all take the same branch and leave together
//   phase B   e -= alpha p, r -= alpha mp (own points only), partial r.r
//   reduce    (second slot, so one barrier per reduction suffices)
//   phase C   p = r + beta p, then a barrier before the next phase A reads
//             neighbours across slab faces
// Values other CTAs of the cluster wrote (p, r, e, mp) are read with ld.cg
// (L2, never a stale L1 line); the scaled coefficients are read-only here.
// A case's vectors (about 13 arrays x 4 or 8 bytes per cell) stay in L2
// across iterations while the cluster lives; finished cases retire and the
// hardware schedules the next cluster.  The loop is bounded by the case's
// iteration cap, and every CTA of a cluster executes the same number of
// barriers, so no barrier can wait forever.
#include "suli_kernels.cuh"

#include <mutex>

#include <cooperative_groups.h>

namespace cgrp = cooperative_groups;

namespace suli {

constexpr int CL_THREADS = 512;
constexpr int CL_MAX = 16;

__device__ __forceinline__ int cbmap(int i, int n, bool per)
{
    if (i < 1) return per ? n : 1;
    if (i > n) return per ? 1 : n;
    return i;
}

// sum of one double per CTA over the cluster; all CTAs get the same value
__device__ __forceinline__ double cluster_sum(cgrp::cluster_group &cl, double v, double *slot, double *shw)
{
    int t = threadIdx.x;
    v = warp_sum(v);
    if ((t & 31) == 0) shw[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        double a = (t < CL_THREADS / 32) ? shw[t] : 0.0;
        a = warp_sum(a);
        if (t == 0) *slot = a;
    }
    cl.sync();
    __shared__ double tot;
    if (t == 0) {
        double s = 0.0;
        const unsigned n = cl.num_blocks();
        for (unsigned r = 0; r < n; ++r) s += *cl.map_shared_rank(slot, r);
        tot = s;
    }
    __syncthreads();
    return tot;
}

template <typename T>
__global__ void __launch_bounds__(CL_THREADS) k_cg_cluster(const CaseDev<T> *__restrict__ cs, int ncases, int mode)
{
    cgrp::cluster_group cl = cgrp::this_cluster();
    const unsigned CL = cl.num_blocks();
    const unsigned rank = cl.block_rank();
    const int cid = blockIdx.x / CL;
    if (cid >= ncases) return;     // whole cluster returns together (same cid)
    const CaseDev<T> &c = cs[cid];
    __shared__ double slots[2];
    __shared__ double shw[CL_THREADS / 32];
    if (c.sc[S_CGACTIVE] == 0.0) return;   // converged / nothing to do: whole cluster agrees
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool px = (c.ccx0 == 0), py = (c.ccy0 == 0);
    const int k0 = 1 + (int)((long long)nz * rank / CL);
    const int k1 = 1 + (int)((long long)nz * (rank + 1) / CL);
    const long long nxy = (long long)nx * ny;
    const long long ncell = nxy * (k1 - k0);
    T *__restrict__ p = c.p;
    T *__restrict__ r = c.r;
    T *__restrict__ e = c.e;
    T *__restrict__ mp = c.mp;
    const T *__restrict__ spi = c.spi;
    const T *__restrict__ spj = c.spj;
    const T *__restrict__ spk = c.spk;
    double rr = c.sc[S_RR];
    const double thr = (mode == 0) ? c.sc[S_THR] : c.sc[S_RRREF];
    const double replay = (mode == 0) ? c.sc[S_CGREPLAY] : -1.0;
    const double cgmax = c.sc[S_CGMAX];
    double it = c.sc[S_CGITER];
    double beta = 0.0;
    bool active = true;
    while (active) {
        // ---- A: mp = A p
        double pm = 0.0;
        for (long long t = threadIdx.x; t < ncell; t += CL_THREADS) {
            int i = 1 + (int)(t % nx);
            long long rem = t / nx;
            int j = 1 + (int)(rem % ny);
            int k = k0 + (int)(rem / ny);
            long long q = g.at(i, j, k);
            T pc = __ldcg(p + q);
            T pxp = (i < nx) ? __ldcg(p + q + 1) : __ldcg(p + g.at(cbmap(nx + 1, nx, px), j, k));
            T pxm = (i > 1) ? __ldcg(p + q - 1) : __ldcg(p + g.at(cbmap(0, nx, px), j, k));
            T pyp = (j < ny) ? __ldcg(p + q + g.sx) : __ldcg(p + g.at(i, cbmap(ny + 1, ny, py), k));
            T pym = (j > 1) ? __ldcg(p + q - g.sx) : __ldcg(p + g.at(i, cbmap(0, ny, py), k));
            T pzp = (k < nz) ? __ldcg(p + q + g.sxy) : pc;
            T pzm = (k > 1) ? __ldcg(p + q - g.sxy) : pc;
            T m = pc - pxp * spi[q + 1] - pxm * spi[q] - pyp * spj[q + g.sx] - pym * spj[q] - pzp * spk[q + g.sxy] -
                  pzm * spk[q];
            __stcg(mp + q, m);
            pm += (double)pc * (double)m;
        }
        double pAp = cluster_sum(cl, pm, &slots[0], shw);
        double alpha = rr / pAp;
        // ---- B: e -= alpha p, r -= alpha mp (points of this thread only)
        double rs = 0.0;
        const T ta = T(alpha);
        for (long long t = threadIdx.x; t < ncell; t += CL_THREADS) {
            int i = 1 + (int)(t % nx);
            long long rem = t / nx;
            int j = 1 + (int)(rem % ny);
            int k = k0 + (int)(rem / ny);
            long long q = g.at(i, j, k);
            T pv = __ldcg(p + q);
            __stcg(e + q, __ldcg(e + q) - ta * pv);
            T rv = __ldcg(r + q) - ta * __ldcg(mp + q);
            __stcg(r + q, rv);
            rs += (double)rv * (double)rv;
        }
        double rrn = cluster_sum(cl, rs, &slots[1], shw);
        beta = rrn / rr;
        rr = rrn;
        it += 1.0;
        if (replay >= 0.0) active = it < replay;
        else active = (fabs(rr) > thr && it < cgmax);
        if (!active) break;
        // ---- C: p = r + beta p
        const T tb = T(beta);
        for (long long t = threadIdx.x; t < ncell; t += CL_THREADS) {
            int i = 1 + (int)(t % nx);
            long long rem = t / nx;
            int j = 1 + (int)(rem % ny);
            int k = k0 + (int)(rem / ny);
            long long q = g.at(i, j, k);
            __stcg(p + q, __ldcg(r + q) + tb * __ldcg(p + q));
        }
        cl.sync();
    }
    // all CTAs keep their shared memory alive until every DSMEM read is done
    cl.sync();
    if (rank == 0 && threadIdx.x == 0) {
        c.sc[S_RR] = rr;
        c.sc[S_BETA] = beta;
        c.sc[S_CGITER] = it;
        c.sc[S_CGACTIVE] = 0.0;
    }
}

// the cluster size of the current device, chosen once per device and element
// type under a lock (handles may be created from several host threads, and
// the devices of one process may differ)
template <typename T>
int cluster_cg_size()
{
    constexpr int kMaxDev = 64;
    static std::mutex mu;
    static int chosen[kMaxDev];
    static bool init = false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
        cudaGetLastError();
        return 0;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!init) {
        for (int d = 0; d < kMaxDev; ++d) chosen[d] = -1;
        init = true;
    }
    if (chosen[dev] >= 0) return chosen[dev];
    int best = 0;
    for (int cl : {16, 8}) {
        cudaFuncSetAttribute(k_cg_cluster<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, cl > 8 ? 1 : 0);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cl, 1, 1);
        cfg.blockDim = dim3(CL_THREADS, 1, 1);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cl;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_cg_cluster<T>, &cfg) == cudaSuccess && nclusters > 0) {
            best = cl;
            break;
        }
        cudaGetLastError();
    }
    chosen[dev] = best;
    return best;
}

// mode 0: the FP64/plain iteration to the case's stop rule; mode 1: one FP32
// pass of the mixed form (stop at the pass target S_RRREF)
template <typename T>
cudaError_t launch_cg_cluster(const Batch<T> &b, int mode, cudaStream_t s)
{
    int cl = cluster_cg_size<T>();
    if (cl == 0) return cudaErrorNotSupported;
    cudaFuncSetAttribute(k_cg_cluster<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, cl > 8 ? 1 : 0);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(cl * b.ncases), 1, 1);
    cfg.blockDim = dim3(CL_THREADS, 1, 1);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    count_launch();
    return cudaLaunchKernelEx(&cfg, k_cg_cluster<T>, (const CaseDev<T> *)b.dcases, b.ncases, mode);
}

template cudaError_t launch_cg_cluster<double>(const Batch<double> &, int, cudaStream_t);
template cudaError_t launch_cg_cluster<float>(const Batch<float> &, int, cudaStream_t);
template int cluster_cg_size<double>();
template int cluster_cg_size<float>();

}  // namespace suli
