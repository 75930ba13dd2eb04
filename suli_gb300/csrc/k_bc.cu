// k_bc.cu -- contorno(nlock) (3_contorno.f90:11-662) as ordered plane fills.
//
// The reference fills whole planes (including edges and corners) in a fixed
// order: pressure ghosts x, y, z (:99-116); velocity ghosts on the y walls,
// the bottom, the top, then the x walls (:118-384); with nlock = 2 the
// wall-normal faces (:394-605).  Edge and corner values depend on that order,
// so each phase is one launch (blockIdx.y = case, threads over the union of
// the plane extents of u, v, w and prd1) and the phases run in sequence:
//   phase 0: prd1 x-ghosts              + velocity y-wall ghosts
//   phase 1: prd1 y-ghosts              + velocity bottom/top ghosts
//   phase 2: prd1 z-ghosts              + velocity x-wall ghosts
//   phase 3 (nlock = 2): wall-normal faces
// Arrays touched in one phase are disjoint from the ones another part of the
// same phase reads, so merging a prd1 phase with a velocity phase is exact.
#include "suli_kernels.cuh"

namespace suli {

#define AT(arr, i, j, k) (arr)[g.at((i), (j), (k))]

// one phase on velocity arrays u, v, w of value type V and (p != nullptr)
// the pressure
template <typename T, typename V>
__device__ __forceinline__ void bc_phase(const CaseDev<T> &c, int phase, V *u, V *v, V *w, V *p)
{
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int nx1 = nx + 1, ny1 = ny + 1, nz1 = nz + 1;
    const bool perx = (c.ccx0 == 0 && c.ccxf == 0);
    const bool pery = (c.ccy0 == 0 && c.ccyf == 0);
    long long nvel, nprd;
    if (phase == 0) { nvel = (long long)(nx + 3) * (nz + 3); nprd = (long long)(ny + 2) * (nz + 2); }
    else if (phase == 1) { nvel = (long long)(nx + 3) * (ny + 3); nprd = (long long)(nx + 2) * (nz + 2); }
    else if (phase == 2) { nvel = (long long)(ny + 3) * (nz + 3); nprd = (long long)(nx + 2) * (ny + 2); }
    else { nvel = (long long)(nx + 2) * (nz + 2) + (long long)(nx + 2) * (ny + 2) + (long long)(ny + 2) * (nz + 2); nprd = 0; }
    if (p == nullptr) nprd = 0;
    const long long ntot = nvel > nprd ? nvel : nprd;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntot; t += (long long)gridDim.x * blockDim.x) {
        // ---- pressure ghosts (:99-116): x in phase 0, y in phase 1, z in phase 2
        if (t < nprd) {
            if (phase == 0) {
                int j = (int)(t % (ny + 2)), k = (int)(t / (ny + 2));
                if (perx) { AT(p, 0, j, k) = AT(p, nx, j, k); AT(p, nx + 1, j, k) = AT(p, 1, j, k); }
                else { AT(p, 0, j, k) = AT(p, 1, j, k); AT(p, nx + 1, j, k) = AT(p, nx, j, k); }
            } else if (phase == 1) {
                int i = (int)(t % (nx + 2)), k = (int)(t / (nx + 2));
                if (pery) { AT(p, i, 0, k) = AT(p, i, ny, k); AT(p, i, ny + 1, k) = AT(p, i, 1, k); }
                else { AT(p, i, 0, k) = AT(p, i, 1, k); AT(p, i, ny + 1, k) = AT(p, i, ny, k); }
            } else {
                int i = (int)(t % (nx + 2)), j = (int)(t / (nx + 2));
                AT(p, i, j, 0) = AT(p, i, j, 1);
                AT(p, i, j, nz + 1) = AT(p, i, j, nz);
            }
        }
        if (t >= nvel) continue;
        if (phase == 0) {
            int i = (int)(t % (nx + 3)), k = (int)(t / (nx + 3));
            bool iu = (i <= nx1 + 1 && k <= nz + 1), iv = (i <= nx + 1 && k <= nz + 1), iw = (i <= nx + 1 && k <= nz1 + 1);
            // y = 0 wall (:118-144)
            if (pery) {
                if (iu) AT(u, i, 0, k) = AT(u, i, ny, k);
                if (iv) AT(v, i, 0, k) = AT(v, i, ny1 - 1, k);
                if (iw) AT(w, i, 0, k) = AT(w, i, ny, k);
            }
            if (c.ccy0 == 1) {
                if (iu) AT(u, i, 0, k) = AT(u, i, 1, k);
                if (iv) AT(v, i, 0, k) = -AT(v, i, 2, k);
                if (iw) AT(w, i, 0, k) = AT(w, i, 1, k);
            }
            if (c.ccy0 == 2) {
                if (iu) AT(u, i, 0, k) = -AT(u, i, 1, k);
                if (iv) AT(v, i, 0, k) = AT(v, i, 2, k);
                if (iw) AT(w, i, 0, k) = -AT(w, i, 1, k);
            }
            // y = ly wall (:146-173)
            if (pery) {
                if (iu) AT(u, i, ny + 1, k) = AT(u, i, 1, k);
                if (iv) AT(v, i, ny1 + 1, k) = AT(v, i, 2, k);
                if (iw) AT(w, i, ny + 1, k) = AT(w, i, 1, k);
            }
            if (c.ccyf == 1) {
                if (iu) AT(u, i, ny + 1, k) = AT(u, i, ny, k);
                if (iv) AT(v, i, ny1 + 1, k) = -AT(v, i, ny1 - 1, k);
                if (iw) AT(w, i, ny + 1, k) = AT(w, i, ny, k);
            }
            if (c.ccyf == 2) {
                if (iu) AT(u, i, ny + 1, k) = -AT(u, i, ny, k);
                if (iv) AT(v, i, ny1 + 1, k) = AT(v, i, ny1 - 1, k);
                if (iw) AT(w, i, ny + 1, k) = -AT(w, i, ny, k);
            }
        } else if (phase == 1) {
            int i = (int)(t % (nx + 3)), j = (int)(t / (nx + 3));
            bool iu = (i <= nx1 + 1 && j <= ny + 1), iv = (i <= nx + 1 && j <= ny1 + 1), iw = (i <= nx + 1 && j <= ny + 1);
            // bottom (:176-196)
            if (c.ccz0 == 1) {
                if (iu) AT(u, i, j, 0) = AT(u, i, j, 1);
                if (iv) AT(v, i, j, 0) = AT(v, i, j, 1);
                if (iw) AT(w, i, j, 0) = -AT(w, i, j, 2);
            }
            if (c.ccz0 == 2) {
                if (iu) AT(u, i, j, 0) = -AT(u, i, j, 1);
                if (iv) AT(v, i, j, 0) = -AT(v, i, j, 1);
                if (iw) AT(w, i, j, 0) = AT(w, i, j, 2);
            }
            // top (:255-275)
            if (c.cczf == 1) {
                if (iu) AT(u, i, j, nz + 1) = AT(u, i, j, nz);
                if (iv) AT(v, i, j, nz + 1) = AT(v, i, j, nz);
                if (iw) AT(w, i, j, nz1 + 1) = -AT(w, i, j, nz1 - 1);
            }
            if (c.cczf == 2) {
                if (iu) AT(u, i, j, nz + 1) = -AT(u, i, j, nz);
                if (iv) AT(v, i, j, nz + 1) = -AT(v, i, j, nz);
                if (iw) AT(w, i, j, nz1 + 1) = AT(w, i, j, nz1 - 1);
            }
        } else if (phase == 2) {
            int j = (int)(t % (ny + 3)), k = (int)(t / (ny + 3));
            bool iu = (j <= ny + 1 && k <= nz + 1), iv = (j <= ny1 + 1 && k <= nz + 1), iw = (j <= ny + 1 && k <= nz1 + 1);
            // x = 0 wall (:278-348)
            if (perx) {
                if (iu) AT(u, 0, j, k) = AT(u, nx1 - 1, j, k);
                if (iv) AT(v, 0, j, k) = AT(v, nx, j, k);
                if (iw) AT(w, 0, j, k) = AT(w, nx, j, k);
            }
            if (c.ccx0 == 1) {
                if (iu) AT(u, 0, j, k) = -AT(u, 2, j, k);
                if (iv) AT(v, 0, j, k) = AT(v, 1, j, k);
                if (iw) AT(w, 0, j, k) = AT(w, 1, j, k);
            }
            if (c.ccx0 == 2) {
                if (iu) AT(u, 0, j, k) = AT(u, 2, j, k);
                if (iv) AT(v, 0, j, k) = -AT(v, 1, j, k);
                if (iw) AT(w, 0, j, k) = -AT(w, 1, j, k);
            }
            if (c.ccx0 == 3) {       // prescribed: v = bxy0 = 0 (2_iniciais.f90:384-385), w = bxz0
                                     // (the waves set it; its plane is one row shorter than w's,
                                     // the top row reads past it upstream: 0 here); u by k_inflow
                if (iv) AT(v, 0, j, k) = V(0.);
                if (iw) AT(w, 0, j, k) = (k <= nz + 1) ? V(c.bxz0[j + (long long)(ny + 3) * k]) : V(0.);
            }
            if (c.ccx0 == 4) {       // validation inflow (:333-348)
                if (iv) AT(v, 0, j, k) = V(0.);
                if (iw) AT(w, 0, j, k) = AT(w, 1, j, k);
            }
            // x = lx wall (:350-384)
            if (perx) {
                if (iu) AT(u, nx1 + 1, j, k) = AT(u, 2, j, k);
                if (iv) AT(v, nx + 1, j, k) = AT(v, 1, j, k);
                if (iw) AT(w, nx + 1, j, k) = AT(w, 1, j, k);
            }
            if (c.ccxf == 1) {
                if (iu) AT(u, nx1 + 1, j, k) = -AT(u, nx1 - 1, j, k);
                if (iv) AT(v, nx + 1, j, k) = AT(v, nx, j, k);
                if (iw) AT(w, nx + 1, j, k) = AT(w, nx, j, k);
            }
            if (c.ccxf == 2) {
                if (iu) AT(u, nx1 + 1, j, k) = AT(u, nx1 - 1, j, k);
                if (iv) AT(v, nx + 1, j, k) = -AT(v, nx, j, k);
                if (iw) AT(w, nx + 1, j, k) = -AT(w, nx, j, k);
            }
            if (c.ccxf == 4) {
                if (iu) AT(u, nx1 + 1, j, k) = AT(u, nx1, j, k);
                if (iv) AT(v, nx + 1, j, k) = AT(v, nx, j, k);
                if (iw) AT(w, nx + 1, j, k) = AT(w, nx, j, k);
            }
        } else {
            // wall-normal faces (:394-605): v over (i,k), w over (i,j), u over (j,k)
            long long nvp = (long long)(nx + 2) * (nz + 2);
            long long nwp = (long long)(nx + 2) * (ny + 2);
            if (t < nvp) {
                int i = (int)(t % (nx + 2)), k = (int)(t / (nx + 2));
                if (pery) AT(v, i, 1, k) = AT(v, i, ny1, k);
                if (c.ccy0 == 1 || c.ccy0 == 2) AT(v, i, 1, k) = V(0.);
                if (pery) AT(v, i, ny1, k) = AT(v, i, 1, k);
                if (c.ccyf == 1 || c.ccyf == 2) AT(v, i, ny1, k) = V(0.);
            } else if (t < nvp + nwp) {
                long long s = t - nvp;
                int i = (int)(s % (nx + 2)), j = (int)(s / (nx + 2));
                if (c.ccz0 == 1 || c.ccz0 == 2 || c.ccz0 == 4) AT(w, i, j, 1) = V(0.);
                if (c.cczf == 1 || c.cczf == 2) AT(w, i, j, nz1) = V(0.);
            } else {
                long long s = t - nvp - nwp;
                int j = (int)(s % (ny + 2)), k = (int)(s / (ny + 2));
                if (perx) AT(u, 1, j, k) = AT(u, nx1, j, k);
                if (c.ccx0 == 1 || c.ccx0 == 2) AT(u, 1, j, k) = V(0.);
                if (perx) AT(u, nx1, j, k) = AT(u, 1, j, k);
                if (c.ccxf == 1 || c.ccxf == 2) AT(u, nx1, j, k) = V(0.);
                if (c.ccxf == 4) AT(u, nx1, j, k) = AT(u, nx1 - 1, j, k);
            }
        }
    }
}

// masters != 0: the same fills on the FP64 masters of the mixed form (after
// they took the values the FP32 fills and the inflow wrote), so that a ghost
// master is the FP64 copy of the master it mirrors, not a rounded one: the
// periodic or wall-symmetric sums that cancel in the pressure equation's
// right-hand side then cancel in FP64 as well
template <typename T>
__global__ void k_bc_phase(const CaseDev<T> *__restrict__ cs, int ncases, int phase, int masters)
{
    const CaseDev<T> &c = cs[blockIdx.y];
    if (masters) {
        if (c.u64 != nullptr) bc_phase<T, double>(c, phase, c.u64, c.v64, c.w64, (double *)nullptr);
    } else {
        bc_phase<T, T>(c, phase, c.u, c.v, c.w, c.prd1);
    }
}

// Prescribed inflow with perturbation (3_contorno.f90:301-330 for I = 0 and
// :532-563 for I = 1).  The reference sweeps k outer, j inner, carrying the
// last water level `iik` across the sweep; one block per case walks the
// levels in that order.  For I = 1 the inflow level set blx1 is imposed on
// ls(1,:,:) first.  Uniform draws come from the counter-based generator
// indexed by (call, j, k), as in the oracle.
template <typename T>
__global__ void k_inflow(const CaseDev<T> *__restrict__ cs, int ncases, int I, double thr_dz,
                         unsigned long long call, int cdev)
{
    if (cdev) call += (unsigned long long)cs[0].sc[S_RNGBASE];
    const CaseDev<T> &c = cs[blockIdx.x];
    if (c.ccx0 != 3) return;
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const unsigned long long base = call * (unsigned long long)ny * (unsigned long long)nz;
    const long long pl = ny + 3;
    T *u = c.u;
    // mixed form: the inflow is formed in FP64 on the masters (velocity and
    // level set) and rounded once into the FP32 copies
    double *u64 = c.u64;
    const bool m = (u64 != nullptr);
    const T *bx = (I == 0) ? c.bxx0 : c.bxx1;
    if (I == 1) {
        for (int t = threadIdx.x; t < ny * nz; t += blockDim.x) {
            int j = 1 + t % ny, k = 1 + t / ny;
            AT(c.ls, 1, j, k) = c.blx1[j + pl * k];
            if (c.ls64 != nullptr) AT(c.ls64, 1, j, k) = (double)c.blx1[j + pl * k];
        }
        __syncthreads();
    }
    // the inflow test on the face level set, (ls(2) + ls(1)) / 2
    auto lsx = [&](int j, int k) -> double {
        if (c.ls64 != nullptr) return (AT(c.ls64, 2, j, k) + AT(c.ls64, 1, j, k)) * 0.5;
        return (double)((AT(c.ls, 2, j, k) + AT(c.ls, 1, j, k)) * T(0.5));
    };
    __shared__ int firstw, lastw;
    if (threadIdx.x == 0) lastw = 0;
    __syncthreads();
    (void)nx;
    for (int k = 1; k <= nz; ++k) {
        if (threadIdx.x == 0) firstw = ny + 1;
        __syncthreads();
        for (int j = 1 + threadIdx.x; j <= ny; j += blockDim.x) {
            if (lsx(j, k) >= -thr_dz * c.dz) atomicMin(&firstw, j);
        }
        __syncthreads();
        for (int j = 1 + threadIdx.x; j <= ny; j += blockDim.x) {
            const double lx = lsx(j, k);
            if (lx >= -thr_dz * c.dz) {
                double r = rng_uniform(c.seed, base + (unsigned long long)((k - 1) * ny + (j - 1)));
                r = 2. * (r - 0.5);
                T v = bx[j + pl * k];
                if (m) {
                    const double x = (double)v * (1. + r * c.iturb);
                    AT(u64, I, j, k) = x;
                    AT(u, I, j, k) = T(x);
                } else {
                    AT(u, I, j, k) = v * (T(1.) + T(r) * T(c.iturb));
                }
            } else if (lx < 0.) {
                int iik = (firstw < j) ? k : lastw;
                if (m) {
                    const double x = AT(u64, I, j, iik) * (1. + tanh(c.pi * (double)(iik - k - 1) / 2.));
                    AT(u64, I, j, k) = x;
                    AT(u, I, j, k) = T(x);
                } else {
                    AT(u, I, j, k) = AT(u, I, j, iik) * (T(1.) + T(tanh(c.pi * (double)(iik - k - 1) / 2.)));
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0 && firstw <= ny) lastw = k;
        __syncthreads();
    }
}

template <typename T>
void launch_contorno(const Batch<T> &b, int nlock, cudaStream_t s, unsigned long long rng_call, int cdev)
{
    if (nlock != 1 && nlock != 2) return;   // nlock = 3 acts only with an IBM (handled by the caller)
    int nb = (b.max_plane + 255) / 256;
    if (nb < 1) nb = 1;
    if (nb > 1024) nb = 1024;
    dim3 grid(nb, b.ncases);
    bool inflow = false;
    for (int c = 0; c < b.ncases; ++c) inflow |= (b.hcases[c].ccx0 == 3);
    // mixed form: every phase runs on the FP32 fields and then on the FP64
    // velocity masters, in the same place relative to the inflow as the FP32
    // fills (the inflow writes both), so a ghost master is the FP64 copy of
    // the master it mirrors at the time the reference copies it
    const bool masters = (sizeof(T) == 4);
    auto phase = [&](int ph) {
        k_bc_phase<T><<<grid, 256, 0, s>>>(b.dcases, b.ncases, ph, 0); count_launch();
        if (masters) { k_bc_phase<T><<<grid, 256, 0, s>>>(b.dcases, b.ncases, ph, 1); count_launch(); }
    };
    for (int ph = 0; ph < 3; ++ph) phase(ph);
    if (inflow) {
        k_inflow<T><<<b.ncases, 256, 0, s>>>(b.dcases, b.ncases, 0, 1.0, rng_call, cdev); count_launch();
    }
    if (nlock == 2) {
        phase(3);
        if (inflow) {
            k_inflow<T><<<b.ncases, 256, 0, s>>>(b.dcases, b.ncases, 1, 2.0, rng_call + 1, cdev); count_launch();
        }
    }
}

// Balanced free outflow (outflow_flux = 1 with ccxf = 4; no counterpart in
// the reference, whose zero-gradient outflow leaves a net boundary flux that
// the all-Neumann pressure equation of graddin cannot absorb): the outflow
// faces u(nx+1, 1:ny, 1:nz) take one uniform correction so that their sum
// equals the inflow faces' u(1, 1:ny, 1:nz).  One 256-thread block per case;
// the plane sum runs in a fixed order (thread t sums q = t, t + 256, ... of
// q = (j-1) + (k-1) ny, then halving pairs in shared memory), so its bits do
// not depend on scheduling.  The mixed form balances the FP64 masters (the
// pressure right-hand side is taken from them) and rounds the faces once.
template <typename T>
__global__ void __launch_bounds__(256) k_outflow_balance(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[blockIdx.x];
    if (c.ccxf != 4 || c.outflow_flux != 1) return;
    const Geo &g = c.g;
    const int ny = g.ny, nz = g.nz, nx1 = g.nx + 1;
    const long long n = (long long)ny * nz;
    __shared__ double sh[256];
    const int t = threadIdx.x;
    double a = 0.0;
    if (c.u64 != nullptr) {
        for (long long q = t; q < n; q += 256) {
            const int j = 1 + (int)(q % ny), k = 1 + (int)(q / ny);
            a += c.u64[g.at(1, j, k)] - c.u64[g.at(nx1, j, k)];
        }
    } else {
        for (long long q = t; q < n; q += 256) {
            const int j = 1 + (int)(q % ny), k = 1 + (int)(q / ny);
            a += (double)c.u[g.at(1, j, k)] - (double)c.u[g.at(nx1, j, k)];
        }
    }
    sh[t] = a;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (t < h) sh[t] += sh[t + h];
        __syncthreads();
    }
    const double corr = sh[0] / (double)n;
    for (long long q = t; q < n; q += 256) {
        const int j = 1 + (int)(q % ny), k = 1 + (int)(q / ny);
        const long long o = g.at(nx1, j, k);
        if (c.u64 != nullptr) {
            const double x = c.u64[o] + corr;
            c.u64[o] = x;
            c.u[o] = T(x);
        } else {
            c.u[o] = T((double)c.u[o] + corr);
        }
    }
}

template <typename T> void launch_outflow_balance(const Batch<T> &b, cudaStream_t s)
{
    bool any = false;
    for (int c = 0; c < b.ncases; ++c) any |= (b.hcases[c].ccxf == 4 && b.hcases[c].outflow_flux == 1);
    if (!any) return;
    k_outflow_balance<T><<<b.ncases, 256, 0, s>>>(b.dcases, b.ncases); count_launch();
}

template void launch_outflow_balance<float>(const Batch<float> &, cudaStream_t);
template void launch_outflow_balance<double>(const Batch<double> &, cudaStream_t);
template void launch_contorno<double>(const Batch<double> &, int, cudaStream_t, unsigned long long, int);
template void launch_contorno<float>(const Batch<float> &, int, cudaStream_t, unsigned long long, int);

}  // namespace suli
