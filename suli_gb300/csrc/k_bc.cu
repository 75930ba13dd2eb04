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

template <typename T>
__global__ void k_bc_phase(const CaseDev<T> *__restrict__ cs, int ncases, int phase)
{
    const CaseDev<T> &c = cs[blockIdx.y];
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int nx1 = nx + 1, ny1 = ny + 1, nz1 = nz + 1;
    T *u = c.u, *v = c.v, *w = c.w, *p = c.prd1;
    const bool perx = (c.ccx0 == 0 && c.ccxf == 0);
    const bool pery = (c.ccy0 == 0 && c.ccyf == 0);
    long long nvel, nprd;
    if (phase == 0) { nvel = (long long)(nx + 3) * (nz + 3); nprd = (long long)(ny + 2) * (nz + 2); }
    else if (phase == 1) { nvel = (long long)(nx + 3) * (ny + 3); nprd = (long long)(nx + 2) * (nz + 2); }
    else if (phase == 2) { nvel = (long long)(ny + 3) * (nz + 3); nprd = (long long)(nx + 2) * (ny + 2); }
    else { nvel = (long long)(nx + 2) * (nz + 2) + (long long)(nx + 2) * (ny + 2) + (long long)(ny + 2) * (nz + 2); nprd = 0; }
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
            if (c.ccx0 == 3) {       // prescribed: bxy0 = bxz0 = 0 (2_iniciais.f90:384-385); u by k_inflow
                if (iv) AT(v, 0, j, k) = T(0.);
                if (iw) AT(w, 0, j, k) = T(0.);
            }
            if (c.ccx0 == 4) {       // validation inflow (:333-348)
                if (iv) AT(v, 0, j, k) = T(0.);
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
                if (c.ccy0 == 1 || c.ccy0 == 2) AT(v, i, 1, k) = T(0.);
                if (pery) AT(v, i, ny1, k) = AT(v, i, 1, k);
                if (c.ccyf == 1 || c.ccyf == 2) AT(v, i, ny1, k) = T(0.);
            } else if (t < nvp + nwp) {
                long long s = t - nvp;
                int i = (int)(s % (nx + 2)), j = (int)(s / (nx + 2));
                if (c.ccz0 == 1 || c.ccz0 == 2 || c.ccz0 == 4) AT(w, i, j, 1) = T(0.);
                if (c.cczf == 1 || c.cczf == 2) AT(w, i, j, nz1) = T(0.);
            } else {
                long long s = t - nvp - nwp;
                int j = (int)(s % (ny + 2)), k = (int)(s / (ny + 2));
                if (perx) AT(u, 1, j, k) = AT(u, nx1, j, k);
                if (c.ccx0 == 1 || c.ccx0 == 2) AT(u, 1, j, k) = T(0.);
                if (perx) AT(u, nx1, j, k) = AT(u, 1, j, k);
                if (c.ccxf == 1 || c.ccxf == 2) AT(u, nx1, j, k) = T(0.);
                if (c.ccxf == 4) AT(u, nx1, j, k) = AT(u, nx1 - 1, j, k);
            }
        }
    }
}

template <typename T>
void launch_contorno(const Batch<T> &b, int nlock, cudaStream_t s)
{
    if (nlock != 1 && nlock != 2) return;   // nlock = 3 acts only with an IBM (handled by the caller)
    int nb = (b.max_plane + 255) / 256;
    if (nb < 1) nb = 1;
    if (nb > 1024) nb = 1024;
    dim3 grid(nb, b.ncases);
    for (int ph = 0; ph < 3; ++ph) k_bc_phase<T><<<grid, 256, 0, s>>>(b.dcases, b.ncases, ph);
    if (nlock == 2) k_bc_phase<T><<<grid, 256, 0, s>>>(b.dcases, b.ncases, 3);
}

template void launch_contorno<double>(const Batch<double> &, int, cudaStream_t);
template void launch_contorno<float>(const Batch<float> &, int, cudaStream_t);

}  // namespace suli
