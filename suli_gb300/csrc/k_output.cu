// k_output.cu -- the field record of PRTSCR (4_plot.f90:501-635) formed on
// the device: velocities averaged to the cell corners, the level set, the
// obstacle's corner level set, and with t_plot = 1 the pressure relative to
// the cell (nx, 1, nz) (prd0 + prd1; prd0 exists with the IPA only), the
// vorticity, nut and ka (zeros without the k equation, as upstream, where
// visco sets ka = 0 and never assigns nut).  Values are formed in FP64 (from the FP64 masters in the mixed form)
// and rounded once to float32, as real(x, 4) does.  The node coordinates are
// written by the host.
#include "suli_kernels.cuh"

namespace suli {

// out (Fortran order, float32): u, v, w at the corners (n1 each), ls at the
// cells (nc), obs_ls at the corners (n1), then with t_plot: p, vort_i,
// vort_j, vort_k, nut, ka at the cells (nc each)
template <typename T>
__global__ void k_prtscr(const CaseDev<T> *__restrict__ cs, int icase, float *__restrict__ out, int t_plot)
{
    const CaseDev<T> &c = cs[icase];
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz, nx1 = nx + 1, ny1 = ny + 1;
    const long long sx = g.sx, sxy = g.sxy;
    const long long n1 = (long long)nx1 * ny1 * (nz + 1), nc = (long long)nx * ny * nz;
    const bool mixed = c.u64 != nullptr;
    auto U = [&](long long q) { return mixed ? c.u64[q] : (double)c.u[q]; };
    auto V = [&](long long q) { return mixed ? c.v64[q] : (double)c.v[q]; };
    auto W = [&](long long q) { return mixed ? c.w64[q] : (double)c.w[q]; };
    float *ua = out, *va = out + n1, *wa = out + 2 * n1, *lso = out + 3 * n1, *obs = lso + nc;
    float *pr = obs + n1, *vi = pr + nc, *vj = vi + nc, *vk = vj + nc, *nut = vk + nc, *ka = nut + nc;
    const long long qref = g.at(nx, 1, nz);
    const double pref = c.prd0 ? (double)c.prd0[qref] + (double)c.prd1[qref] : (double)c.prd1[qref];
    const long long n = n1 > nc ? n1 : nc;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        if (t < n1) {       // corner (i, j, k), 1..nx1 x 1..ny1 x 1..nz1 (4_plot.f90:556-566)
            const int i = 1 + (int)(t % nx1);
            const long long r = t / nx1;
            const int j = 1 + (int)(r % ny1), k = 1 + (int)(r / ny1);
            const long long q = g.at(i, j, k);
            ua[t] = (float)((U(q) + U(q - sx) + U(q - sxy) + U(q - sx - sxy)) * 0.25);
            va[t] = (float)((V(q) + V(q - 1) + V(q - sxy) + V(q - 1 - sxy)) * 0.25);
            wa[t] = (float)((W(q) + W(q - sx) + W(q - 1) + W(q - 1 - sx)) * 0.25);
            obs[t] = (c.obst_t == 0) ? 0.0f : (float)c.obs_ls[q];
        }
        if (t < nc) {       // cell (i, j, k), 1..nx x 1..ny x 1..nz
            const int i = 1 + (int)(t % nx);
            const long long r = t / nx;
            const int j = 1 + (int)(r % ny), k = 1 + (int)(r / ny);
            const long long q = g.at(i, j, k);
            lso[t] = (float)(mixed ? c.ls64[q] : (double)c.ls[q]);
            if (t_plot) {
                pr[t] = (float)((c.prd0 ? (double)c.prd0[q] + (double)c.prd1[q] : (double)c.prd1[q]) - pref);
                const double dudy = (U(q + sx) - U(q)) * c.idy, dudz = (U(q + sxy) - U(q)) * c.idz;
                const double dvdx = (V(q + 1) - V(q)) * c.idx, dvdz = (V(q + sxy) - V(q)) * c.idz;
                const double dwdx = (W(q + 1) - W(q)) * c.idx, dwdy = (W(q + sx) - W(q)) * c.idy;
                vi[t] = (float)(dwdy - dvdz);
                vj[t] = (float)(dudz - dwdx);
                vk[t] = (float)(dvdx - dudy);
                nut[t] = c.nut ? (float)c.nut[q] : 0.0f;
                ka[t] = c.ka ? (float)c.ka[q] : 0.0f;
            }
        }
    }
}

template <typename T> void launch_prtscr(const Batch<T> &b, int icase, float *out, int t_plot, cudaStream_t s)
{
    static const int grid = occupancy_grid((const void *)k_prtscr<T>);
    k_prtscr<T><<<grid, 256, 0, s>>>(b.dcases, icase, out, t_plot);
    count_launch();
}

template void launch_prtscr<float>(const Batch<float> &, int, float *, int, cudaStream_t);
template void launch_prtscr<double>(const Batch<double> &, int, float *, int, cudaStream_t);

}  // namespace suli
