// k_momentum.cu -- momentum-side kernels.
//
//   k_visco_mu      5_viscosidade.f90:11-151  Smagorinsky mu_t, mu = ls_mu + mu_t
//                   (m_turb >= 2: the strain sum for the k equation of k_keq.cu)
//   k_visco_faces   5_viscosidade.f90:153-155 mu -> xmu/ymu/zmu (interp*_cf)
//   k_convdiff      6_convdiff.f90:14-167 with classico der=3 (7_advectivo.f90:171-284);
//                   optionally fused with complementos (11_diversos.f90:355-450)
//   k_tempo         11_diversos.f90:10-296
//   k_posdin        10_pos.f90:1-46
//   k_conmassa      4_plot.f90:386-394 (FP64 divergence and max|div|)
//   k_mms_error     13_mms.f90:391-451
//
// One thread per (i,j,k) handles the u, v and w locations that exist there,
// so Fu/Fv/Fw (and the u/v/w updates) come from one launch.  The reference's
// temporaries (advecting-velocity averages, interpolated viscosities, face
// densities, upwind derivatives) are recomputed in registers with the same
// operations and boundary copies as the Fortran helpers.
#include "conv_faces.cuh"

namespace suli {

#define AT(arr, i, j, k) (arr)[g.at((i), (j), (k))]

// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_visco_mu(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    long long q = g.at(i, j, k);
    T mut = T(0.);
    if (c.m_turb >= 1) {
        const T *u = c.u, *v = c.v, *w = c.w;
        const T tdx = T(1.0 / (2. * c.dx)), tdy = T(1.0 / (2. * c.dy)), tdz = T(1.0 / (2. * c.dz));
        // derivax/y/z on the staggered arrays then interp?_fc to the centre
        T dudx = ((AT(u, i + 1, j, k) - AT(u, i - 1, j, k)) * tdx + (AT(u, i + 2, j, k) - AT(u, i, j, k)) * tdx) * T(0.5);
        T dudy = ((AT(u, i, j + 1, k) - AT(u, i, j - 1, k)) * tdy + (AT(u, i + 1, j + 1, k) - AT(u, i + 1, j - 1, k)) * tdy) * T(0.5);
        T dudz = ((AT(u, i, j, k + 1) - AT(u, i, j, k - 1)) * tdz + (AT(u, i + 1, j, k + 1) - AT(u, i + 1, j, k - 1)) * tdz) * T(0.5);
        T dvdx = ((AT(v, i + 1, j, k) - AT(v, i - 1, j, k)) * tdx + (AT(v, i + 1, j + 1, k) - AT(v, i - 1, j + 1, k)) * tdx) * T(0.5);
        T dvdy = ((AT(v, i, j + 1, k) - AT(v, i, j - 1, k)) * tdy + (AT(v, i, j + 2, k) - AT(v, i, j, k)) * tdy) * T(0.5);
        T dvdz = ((AT(v, i, j, k + 1) - AT(v, i, j, k - 1)) * tdz + (AT(v, i, j + 1, k + 1) - AT(v, i, j + 1, k - 1)) * tdz) * T(0.5);
        T dwdx = ((AT(w, i + 1, j, k) - AT(w, i - 1, j, k)) * tdx + (AT(w, i + 1, j, k + 1) - AT(w, i - 1, j, k + 1)) * tdx) * T(0.5);
        T dwdy = ((AT(w, i, j + 1, k) - AT(w, i, j - 1, k)) * tdy + (AT(w, i, j + 1, k + 1) - AT(w, i, j - 1, k + 1)) * tdy) * T(0.5);
        T dwdz = ((AT(w, i, j, k + 1) - AT(w, i, j, k - 1)) * tdz + (AT(w, i, j, k + 2) - AT(w, i, j, k)) * tdz) * T(0.5);
        T p1 = dudx + T(0.5) * (dudy + dvdx + dudz + dwdx);
        T p2 = dvdy + T(0.5) * (dvdx + dudy + dvdz + dwdy);
        T p3 = dwdz + T(0.5) * (dwdy + dvdz + dudz + dwdx);
        const T sm = p1 + p2 + p3;
        if (c.m_turb >= 2) {   // the k equation's production term uses it (:117-122); mut comes after its loop
            c.sij[q] = sm;
            return;
        }
        mut = T(c.cles) * sqrt(T(2.) * sm * sm) * c.rho[q];
    }
    c.mut[q] = mut;
    c.mu[q] = c.ls_mu[q] + mut;
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_visco_faces(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const T *mu = c.mu;
    bool px = (c.ccx0 == 0);
    if (i <= nx + 1 && j <= ny && k <= nz)
        AT(c.xmu, i, j, k) = interp_cf<T>(i, nx, px, [&](int m) { return AT(mu, m, j, k); });
    if (i <= nx && j <= ny + 1 && k <= nz)
        AT(c.ymu, i, j, k) = interp_cf<T>(j, ny, false, [&](int m) { return AT(mu, i, m, k); });
    if (i <= nx && j <= ny && k <= nz + 1) {
        auto get = [&](int m) { return AT(mu, i, j, m); };
        AT(c.zmu, i, j, k) = c.dzk ? zcf_w<T>(c, k, nz, get) : interp_cf<T>(k, nz, false, get);   // SuLi-ICdz/5_viscosidade.f90:155
    }
}

// ---------------------------------------------------------------------------
// the gather form (operands read from global memory, one thread per
// (i, j, k)); the FP64 form's default and the fallback SULI_CONVDIFF=0
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_convdiff(const CaseDev<T> *__restrict__ cs, int ncases, int fuse)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const GlobalAcc<T> X{c};
    const bool vz = (c.dzk != nullptr);   // SuLi-ICdz's variable z spacing
    if (i <= nx + 1 && j <= ny && k <= nz) {
        T F = vz ? face_fu<T, GlobalAcc<T>, false, true>(c, X, i, j, k) : face_fu<T>(c, X, i, j, k);
        if (fuse) F = compl_fu<T>(c, F, i, j, k);
        AT(c.Fu, i, j, k) = F;
    }
    if (i <= nx && j <= ny + 1 && k <= nz) {
        T F = vz ? face_fv<T, GlobalAcc<T>, false, true>(c, X, i, j, k) : face_fv<T>(c, X, i, j, k);
        if (fuse) F = compl_fv<T>(c, F, i, j, k);
        AT(c.Fv, i, j, k) = F;
    }
    if (i <= nx && j <= ny && k <= nz + 1) {
        T F = vz ? face_fw<T, GlobalAcc<T>, false, true>(c, X, i, j, k) : face_fw<T>(c, X, i, j, k);
        if (fuse) F = compl_fw<T>(c, F, AT(c.w, i, j, k), i, j, k);
        AT(c.Fw, i, j, k) = F;
    }
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_complementos(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    // the surface-tension term sits between gravity and the MMS source, the
    // kinetic-energy term (m_turb >= 2) comes last
    const bool ten = (c.t_tens == 1), kt = (c.m_turb >= 2);
    if (i <= nx + 1 && j <= ny && k <= nz) {
        T F = AT(c.Fu, i, j, k) + T(c.gx);
        if (ten) F = F - tension_face(c, 0, i, j, k);
        F = F + AT(c.tf_u, i, j, k);
        if (kt) F = F - ka_face(c, 0, i, j, k);
        AT(c.Fu, i, j, k) = F;
    }
    if (i <= nx && j <= ny + 1 && k <= nz) {
        T F = AT(c.Fv, i, j, k);
        if (ten) F = F - tension_face(c, 1, i, j, k);
        F = F + AT(c.tf_v, i, j, k);
        if (kt) F = F - ka_face(c, 1, i, j, k);
        AT(c.Fv, i, j, k) = F;
    }
    if (i <= nx && j <= ny && k <= nz + 1) {
        T F = AT(c.Fw, i, j, k) - T(c.gz);
        if (c.epis) F = F - (AT(c.w, i, j, k) - T(0.)) * AT(c.epis, i, j, k);
        if (ten) F = F - tension_face(c, 2, i, j, k);
        F = F + AT(c.tf_w, i, j, k);
        if (kt) F = F - ka_face(c, 2, i, j, k);
        AT(c.Fw, i, j, k) = F;
    }
}

// ---------------------------------------------------------------------------
// sponge_layer (3_contorno.f90:1011-1103), called by complementos: epis_z on
// the w faces of the columns i >= nint(x_inicial / dx) + 1 (x_inicial = nx dx
// - 1 m; clamped to 1), in FP64 and stored once rounded.  esp_type 1 grades
// it with the interface height zpfs(i) of the last (j, k) of the plane where
// ls changes sign (a block max-reduction of the loop index; no sign change:
// the domain height when the plane's first cell is water, else 0, for the
// value the reference leaves unset); the heights z_x are the reference's
// running sums.  Grid: x = column i - 1, y = case.
template <typename T>
__global__ void __launch_bounds__(256) k_sponge(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[blockIdx.y];
    if (c.esp_type <= 0) return;
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int i = blockIdx.x + 1;
    if (i > nx) return;
    const double dx = c.dx, dz = c.dz;
    const double l_sponge = 1., x_inicial = nx * dx - l_sponge;
    const double alfa = 60., alfa0 = 0., alfa1 = 30.;
    int i0 = (int)llround(x_inicial / dx) + 1;
    if (i0 < 1) i0 = 1;
    if (i < i0) return;
    const double zpt = dz * nz;
    // the level set in FP64: the mixed form's FP64 master (an FP32 product of
    // two small values near the interface can underflow to 0 and count as a
    // crossing), else the FP64 field itself
    auto lsd = [&](int a, int bb, int d) -> double {
        const long long q = g.at(a, bb, d);
        return c.ls64 != nullptr ? c.ls64[q] : (double)c.ls[q];
    };
    __shared__ long long red[32];
    __shared__ double zpfs_s;
    if (c.esp_type == 1) {
        long long best = -1;
        const long long nk = nz - 1, n = (long long)ny * nk;
        for (long long t = threadIdx.x; t < n; t += blockDim.x) {
            const int j = (int)(t / nk) + 1, k = (int)(t % nk) + 1;
            if (lsd(i, j, k) * lsd(i, j, k + 1) <= 0.) best = t;   // t grows per thread
        }
        for (int o = 16; o > 0; o >>= 1) {
            const long long v = __shfl_down_sync(0xffffffffu, best, o);
            best = v > best ? v : best;
        }
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            long long b = -1;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = red[w] > b ? red[w] : b;
            double z = (lsd(i, 1, 1) >= 0.) ? zpt : 0.;
            if (b >= 0) {
                const int j = (int)(b / nk) + 1, k = (int)(b % nk) + 1;
                const double alt1 = dz * (k - 0.5) + lsd(i, j, k);
                const double alt2 = dz * (k + 0.5) + lsd(i, j, k + 1);
                z = alt1 > alt2 ? alt1 : alt2;
            }
            zpfs_s = z;
        }
        __syncthreads();
    }
    const double zpfs = (c.esp_type == 1) ? zpfs_s : 0.;
    const double xp = (i - 0.5) * dx;
    const double aux1 = (xp - x_inicial) / l_sponge;
    for (int j = 1 + threadIdx.x; j <= ny; j += blockDim.x) {
        double zx = -dz;
        for (int k = 1; k <= nz; ++k) {
            zx = zx + dz;
            double e;
            if (c.esp_type == 1) {
                if (lsd(i, j, k) >= 0.) e = alfa * aux1 * aux1 * (0. - zx) / (0. - zpfs);
                else e = alfa * aux1 * aux1 * (zx - zpt) / (zpfs - zpt);
            } else {
                e = alfa0 + aux1 * (alfa1 - alfa0);
            }
            AT(c.epis, i, j, k) = T(e);
        }
    }
}

// ---------------------------------------------------------------------------
// tempo (11_diversos.f90:10-296) at one location
template <typename T>
__device__ __forceinline__ void tempo_one(const CaseDev<T> &c, int tt, int it, T dt, long long q, T *u, const T *F, T *u0,
                                          T *f0, T *f1)
{
    const int tte = c.t_tempo;
    T Fv = F[q];
    if ((tte == 0) || ((tte == 3) || ((tte == 4) && (it == 1)))) {
        u[q] = u[q] + dt * Fv;
        if (tte == 3 || tte == 4) f0[q] = Fv;
    } else if (tte == 1) {
        if (tt == 1) { u0[q] = u[q]; u[q] = u[q] + dt * Fv; }
        else if (tt == 2) { u[q] = u0[q] + dt * Fv; }
    } else if (tte == 2) {
        if (tt == 1) {
            u0[q] = u[q]; f0[q] = Fv; u[q] = u[q] + dt * Fv;
        } else if (tt == 2) {
            T aux1 = T(2.) * dt;
            f1[q] = Fv;
            u[q] = u0[q] - dt * f0[q] + aux1 * Fv;
        } else if (tt == 3) {
            T aux1 = dt / T(6.);
            u[q] = u0[q] + aux1 * (f0[q] + T(4.) * f1[q] + Fv);
        }
    } else if (((tte == 3) && (it != 1)) || ((tte == 4) && (it == 2))) {
        u[q] = u[q] + dt * T(0.5) * (3 * Fv - f0[q]);
        f0[q] = Fv;
        if (tte == 4) f1[q] = f0[q];
    } else if ((tte == 4) && (it >= 3)) {
        T aux1 = dt / T(12.);
        u[q] = u[q] + aux1 * (T(23.) * Fv - T(16.) * f0[q] + T(5.) * f1[q]);
        f1[q] = f0[q];
        f0[q] = Fv;
    }
}

// the same update on the FP64 masters of the mixed form (u = master, u0 =
// its stage copy; F, f0, f1 stay FP32); the FP32 copies follow the masters
template <typename T>
__device__ __forceinline__ void tempo_one_m(const CaseDev<T> &c, int tt, int it, const T (&dtv)[4], long long q, T *u,
                                            double *um, const T *F, T *u0, double *u0m, T *f0, T *f1)
{
    // the increment of the scheme from the FP32 tendencies in FP32 (dt F is
    // small against u: its FP32 rounding is far below the master's), added
    // to the FP64 master: one widening, one FP64 add and one rounding per
    // component on GB300's FP64 pipe; dtv = dt, dt/6, dt/2, dt/12 rounded
    // to FP32 (formed once per block)
    const int tte = c.t_tempo;
    const T Fv = F[q];
    const T dtf = dtv[0];
    double x = um[q];
    if ((tte == 0) || ((tte == 3) || ((tte == 4) && (it == 1)))) {
        x = x + (double)(dtf * Fv);
        if (tte == 3 || tte == 4) f0[q] = Fv;
    } else if (tte == 1) {
        if (tt == 1) { u0m[q] = x; u0[q] = T(x); x = x + (double)(dtf * Fv); }
        else if (tt == 2) { x = u0m[q] + (double)(dtf * Fv); }
    } else if (tte == 2) {
        if (tt == 1) {
            u0m[q] = x; u0[q] = T(x); f0[q] = Fv; x = x + (double)(dtf * Fv);
        } else if (tt == 2) {
            f1[q] = Fv;
            x = u0m[q] + (double)(dtf * (T(2) * Fv - f0[q]));
        } else if (tt == 3) {
            x = u0m[q] + (double)(dtv[1] * (f0[q] + T(4) * f1[q] + Fv));
        }
    } else if (((tte == 3) && (it != 1)) || ((tte == 4) && (it == 2))) {
        x = x + (double)(dtv[2] * (T(3) * Fv - f0[q]));
        f0[q] = Fv;
        if (tte == 4) f1[q] = f0[q];
    } else if ((tte == 4) && (it >= 3)) {
        x = x + (double)(dtv[3] * (T(23) * Fv - T(16) * f0[q] + T(5) * f1[q]));
        f1[q] = f0[q];
        f0[q] = Fv;
    }
    um[q] = x;
    u[q] = T(x);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_tempo(const CaseDev<T> *__restrict__ cs, int ncases, int tt, int it)
{
    if (it < 0) it = (int)cs[0].sc[S_ITSTEP];
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    // mixed form: the scheme's FP32 step factors, formed once per block (a
    // per-thread FP64 divide by 6 or 12 is a long sequence on GB300's FP64 pipe)
    __shared__ T s_dt[4];
    if (c.u64 != nullptr) {
        if (tid_lin() == 0) {
            const double dt = c.sc[S_DT];
            s_dt[0] = T(dt); s_dt[1] = T(dt / 6.); s_dt[2] = T(dt * 0.5); s_dt[3] = T(dt / 12.);
        }
        __syncthreads();
    }
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    long long q = g.at(i, j, k);
    if (c.ipa) {   // the IPA's explicit pressure force first (:21-45), kept in F as upstream
        if (i <= nx + 1 && j <= ny && k <= nz) c.Fu[q] = c.Fu[q] + c.px[q];
        if (i <= nx && j <= ny + 1 && k <= nz) c.Fv[q] = c.Fv[q] + c.py[q];
        if (i <= nx && j <= ny && k <= nz + 1) c.Fw[q] = c.Fw[q] + c.pz[q];
    }
    if (c.u64 != nullptr) {
        const T dtv[4] = {s_dt[0], s_dt[1], s_dt[2], s_dt[3]};
        if (i <= nx + 1 && j <= ny && k <= nz) tempo_one_m<T>(c, tt, it, dtv, q, c.u, c.u64, c.Fu, c.u0, c.u064, c.fu0, c.fu1);
        if (i <= nx && j <= ny + 1 && k <= nz) tempo_one_m<T>(c, tt, it, dtv, q, c.v, c.v64, c.Fv, c.v0, c.v064, c.fv0, c.fv1);
        if (i <= nx && j <= ny && k <= nz + 1) tempo_one_m<T>(c, tt, it, dtv, q, c.w, c.w64, c.Fw, c.w0, c.w064, c.fw0, c.fw1);
        return;
    }
    T dt = T(c.sc[S_DT]);
    if (i <= nx + 1 && j <= ny && k <= nz) tempo_one<T>(c, tt, it, dt, q, c.u, c.Fu, c.u0, c.fu0, c.fu1);
    if (i <= nx && j <= ny + 1 && k <= nz) tempo_one<T>(c, tt, it, dt, q, c.v, c.Fv, c.v0, c.fv0, c.fv1);
    if (i <= nx && j <= ny && k <= nz + 1) tempo_one<T>(c, tt, it, dt, q, c.w, c.Fw, c.w0, c.fw0, c.fw1);
}

// FP32 velocity and level-set values written outside the FP64 updates
// (boundary fills, inflow, IBM images) -> FP64 masters: an element whose FP32
// copy no longer equals its rounded master takes the FP32 value.  Grid: x
// strides the case's box, y = case.
template <typename T>
__global__ void k_sync_masters(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[blockIdx.y];
    if (c.u64 == nullptr) return;
    // contorno's plane fills run on the masters in FP64 and the inflow
    // writes them too; the FP32 writes left to copy are the IBM image points
    // (anywhere in the box; before the plane fills) and, for callers that
    // run it after contorno, the inflow planes i = 0 and 1
    const bool ibm = (c.obst_t != 0 && c.ibm_t == 2);
    if (!ibm && c.ccx0 != 3) return;
    const long long rows = c.g.sxy / c.g.sx * (long long)(c.g.nz + 3);
    const long long n = ibm ? c.g.total : 2 * rows;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long q = ibm ? t : (t % 2) + c.g.sx * (t / 2);
        const T u = c.u[q], v = c.v[q], w = c.w[q], l = c.ls[q];
        if (T(c.u64[q]) != u) c.u64[q] = (double)u;
        if (T(c.v64[q]) != v) c.v64[q] = (double)v;
        if (T(c.w64[q]) != w) c.w64[q] = (double)w;
        if (T(c.ls64[q]) != l) c.ls64[q] = (double)l;
    }
}

// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_posdin(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const T *p = c.prd1;
    const T *rho = c.rho;
    T dt = T(c.sc[S_DT]);
    T aux1 = dt / T(c.dx), aux2 = dt / T(c.dy);
    bool px = (c.ccx0 == 0);
    const bool py = (c.ccy0 == 0);
    // pressure difference across a face: in the mixed form from the FP64
    // pressure of the last solve when it is current (the FP32 pressure loses
    // a digit to cancellation where the hydrostatic part dominates); ghost
    // indices map to the interior cell their Neumann copy / periodic wrap holds
    const bool p64 = (sizeof(T) == 4) && c.e64 != nullptr && c.sc[S_P64OK] != 0.0;
    auto dp = [&](int i1, int j1, int k1, int i0, int j0, int k0) -> T {
        if (!p64) return AT(p, i1, j1, k1) - AT(p, i0, j0, k0);
        auto mi = [&](int a) { return a < 1 ? (px ? nx : 1) : (a > nx ? (px ? 1 : nx) : a); };
        auto mj = [&](int a) { return a < 1 ? (py ? ny : 1) : (a > ny ? (py ? 1 : ny) : a); };
        auto mk = [&](int a) { return a < 1 ? 1 : (a > nz ? nz : a); };
        return T(c.e64[g.at(mi(i1), mj(j1), mk(k1))] - c.e64[g.at(mi(i0), mj(j0), mk(k0))]);
    };
    if (c.u64 != nullptr) {
        // mixed form: the whole correction in FP64 on the masters, with the
        // density the FP64 pressure operator was built from (rho64), so the
        // projection stays consistent with the solve
        const double ddt = c.sc[S_DT];
        const double *r64 = c.rho64;
        auto dp64 = [&](int i1, int j1, int k1, int i0, int j0, int k0) -> double {
            auto mi = [&](int a) { return a < 1 ? (px ? nx : 1) : (a > nx ? (px ? 1 : nx) : a); };
            auto mj = [&](int a) { return a < 1 ? (py ? ny : 1) : (a > ny ? (py ? 1 : ny) : a); };
            auto mk = [&](int a) { return a < 1 ? 1 : (a > nz ? nz : a); };
            if (p64) return c.e64[g.at(mi(i1), mj(j1), mk(k1))] - c.e64[g.at(mi(i0), mj(j0), mk(k0))];
            return (double)AT(p, i1, j1, k1) - (double)AT(p, i0, j0, k0);
        };
        // the face factor dt / (h rho_face): dt times the unit factor the
        // solve's operator stored, when its pressure is current, else formed
        // here (by reciprocal: no FP64 divide, a long sequence on GB300's
        // FP64 units)
        auto factor = [&](const double *pf, long long q, double ih, double rf) {
            return p64 ? ddt * pf[q] : (ddt * ih) * rcp_nr64(rf);
        };
        if (i <= nx + 1 && j <= ny && k <= nz) {
            const long long q = g.at(i, j, k);
            const double f = factor(c.pfx64, q, c.idx, p64 ? 1.0 : interp_cf<double>(i, nx, px, [&](int m) { return AT(r64, m, j, k); }));
            const double x = c.u64[q] - dp64(i, j, k, i - 1, j, k) * f;
            c.u64[q] = x;
            c.u[q] = T(x);
        }
        if (i <= nx && j <= ny + 1 && k <= nz) {
            const long long q = g.at(i, j, k);
            const double f = factor(c.pfy64, q, c.idy, p64 ? 1.0 : interp_cf<double>(j, ny, false, [&](int m) { return AT(r64, i, m, k); }));
            const double x = c.v64[q] - dp64(i, j, k, i, j - 1, k) * f;
            c.v64[q] = x;
            c.v[q] = T(x);
        }
        if (i <= nx && j <= ny && k <= nz + 1) {
            const long long q = g.at(i, j, k);
            double f;
            if (c.dzk && !p64) {   // SuLi-ICdz/10_pos.f90:41: dt / dzz(k) over the spacing-weighted face density
                const int ff = k < 2 ? 2 : (k > nz ? nz : k);
                const double a = c.dzk[ff], b = c.dzk[ff - 1];
                f = (ddt * c.idzzk[k]) * rcp_nr64((AT(r64, i, j, ff) * a + AT(r64, i, j, ff - 1) * b) / (a + b));
            } else {
                f = factor(c.pfz64, q, c.idz, p64 ? 1.0 : interp_cf<double>(k, nz, false, [&](int m) { return AT(r64, i, j, m); }));
            }
            const double x = c.w64[q] - dp64(i, j, k, i, j, k - 1) * f;
            c.w64[q] = x;
            c.w[q] = T(x);
        }
        return;
    }
    if (i <= nx + 1 && j <= ny && k <= nz) {
        T rx = interp_cf<T>(i, nx, px, [&](int m) { return AT(rho, m, j, k); });
        AT(c.u, i, j, k) = AT(c.u, i, j, k) - aux1 * dp(i, j, k, i - 1, j, k) / rx;
    }
    if (i <= nx && j <= ny + 1 && k <= nz) {
        T ry = interp_cf<T>(j, ny, false, [&](int m) { return AT(rho, i, m, k); });
        AT(c.v, i, j, k) = AT(c.v, i, j, k) - aux2 * dp(i, j, k, i, j - 1, k) / ry;
    }
    if (i <= nx && j <= ny && k <= nz + 1) {
        auto get = [&](int m) { return AT(rho, i, j, m); };
        if (c.dzk) {   // SuLi-ICdz/10_pos.f90:41
            T rz = zcf_w<T>(c, k, nz, get);
            AT(c.w, i, j, k) = AT(c.w, i, j, k) - dt / T(c.dzzk[k]) * dp(i, j, k, i, j, k - 1) / rz;
        } else {
            T rz = interp_cf<T>(k, nz, false, get);
            AT(c.w, i, j, k) = AT(c.w, i, j, k) - dt / T(c.dz) * dp(i, j, k, i, j, k - 1) / rz;
        }
    }
}

// divergence in FP64 (also in the mixed form) and its maximum
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_conmassa(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    double m = 0.0;
    if (i <= g.nx && j <= g.ny && k <= g.nz) {
        double d;
        if (c.u64 != nullptr) {   // mixed form: the FP64 masters
            const double *u = c.u64, *v = c.v64, *w = c.w64;
            d = (AT(u, i + 1, j, k) - AT(u, i, j, k)) * c.idx + (AT(v, i, j + 1, k) - AT(v, i, j, k)) * c.idy +
                (AT(w, i, j, k + 1) - AT(w, i, j, k)) * (c.dzk ? c.idzzk[k] : c.idz);
        } else {
            const T *u = c.u, *v = c.v, *w = c.w;
            d = ((double)AT(u, i + 1, j, k) - (double)AT(u, i, j, k)) / c.dx +
                ((double)AT(v, i, j + 1, k) - (double)AT(v, i, j, k)) / c.dy +
                ((double)AT(w, i, j, k + 1) - (double)AT(w, i, j, k)) / (c.dzk ? c.dzzk[k] : c.dz);   // SuLi-ICdz/4_plot.f90:406
        }
        AT(c.div, i, j, k) = T(d);
        m = fabs(d);
        if (!(m <= 1.79769313486231570e308)) m = INFINITY;   // NaN counts as infinite: fmax would drop it
    }
    double vals[1] = {m}, tot[1];
    if (last_block_reduce<T, 1>(c, vals, tot, 1u) && tid_lin() == 0) c.sc[S_MAXDIV] = tot[0];
}

// masked RMS errors against the steady manufactured fields (a = 0: w_m = 0, p_m = 0)
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_mms_error(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const T *ls = c.ls;
    bool px = (c.ccx0 == 0);
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const double pi = c.pi, h = 2.0;
    if (i <= nx + 1 && j <= ny && k <= nz) {
        T lx = interp_cf<T>(i, nx, px, [&](int m) { return AT(ls, m, j, k); });
        if (lx > T(0.)) {
            double x = (i - 1.0) * c.dx, y = (j - 0.5) * c.dy, z = (k - 0.5) * c.dz;
            double um = sin(x) * cos(y) * sin(pi * 0.5 * z / h) - cos(x) * sin(y) * (cos(pi * 2. * z / h) - 1.);
            double d = um - (double)AT(c.u, i, j, k);
            s[0] = d * d; s[4] = 1.0;
        }
    }
    if (i <= nx && j <= ny + 1 && k <= nz) {
        T ly = interp_cf<T>(j, ny, false, [&](int m) { return AT(ls, i, m, k); });
        if (ly > T(0.)) {
            double x = (i - 0.5) * c.dx, y = (j - 1.0) * c.dy, z = (k - 0.5) * c.dz;
            double vm = -cos(x) * sin(y) * sin(pi * 0.5 * z / h) + sin(x) * cos(y) * (cos(pi * 2. * z / h) - 1.);
            double d = vm - (double)AT(c.v, i, j, k);
            s[1] = d * d; s[5] = 1.0;
        }
    }
    if (i <= nx && j <= ny && k <= nz + 1) {
        T lz = interp_cf<T>(k, nz, false, [&](int m) { return AT(ls, i, j, m); });
        if (lz > T(0.)) {
            double d = (double)AT(c.w, i, j, k);
            s[2] = d * d; s[6] = 1.0;
        }
    }
    if (i <= nx && j <= ny && k <= nz) {
        if (AT(ls, i, j, k) > T(0.)) {
            double d = (double)AT(c.prd1, i, j, k);
            s[3] = d * d; s[7] = 1.0;
        }
    }
    double tot[8];
    if (last_block_reduce<T, 8>(c, s, tot) && tid_lin() == 0) {
        c.sc[S_ERR0] = sqrt(tot[0] / fmax(tot[4], 1.0));
        c.sc[S_ERR1] = sqrt(tot[1] / fmax(tot[5], 1.0));
        c.sc[S_ERR2] = sqrt(tot[2] / fmax(tot[6], 1.0));
        c.sc[S_ERR3] = sqrt(tot[3] / fmax(tot[7], 1.0));
    }
}

template <typename T>
__global__ void k_set_scalar(const CaseDev<T> *__restrict__ cs, int ncases, int slot, double v)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < ncases) cs[q].sc[slot] = v;
}

// ---- launchers -------------------------------------------------------------
template <typename T> void launch_visco(const Batch<T> &b, int keq_stages, const double *a_dt, cudaStream_t s)
{
    k_visco_mu<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    if (keq_stages > 0) launch_keq<T>(b, keq_stages, a_dt, s);   // m_turb >= 2 cases
    k_visco_faces<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
template <typename T> void launch_sponge(const Batch<T> &b, cudaStream_t s)
{
    int nxmax = 1;
    bool any = false;
    for (int c = 0; c < b.ncases; ++c) {
        nxmax = b.hcases[c].g.nx > nxmax ? b.hcases[c].g.nx : nxmax;
        any |= b.hcases[c].esp_type > 0;
    }
    if (!any) return;
    k_sponge<T><<<dim3(nxmax, b.ncases), 256, 0, s>>>(b.dcases, b.ncases); count_launch();
}
template <typename T> void launch_convdiff(const Batch<T> &b, int fuse, cudaStream_t s)
{
    k_convdiff<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, fuse); count_launch();
}

template <typename T> void launch_complementos(const Batch<T> &b, cudaStream_t s)
{
    k_complementos<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
template <typename T> void launch_tempo(const Batch<T> &b, int tt, int it, cudaStream_t s)
{
    k_tempo<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, tt, it); count_launch();
}
template <typename T> void launch_sync_masters(const Batch<T> &b, cudaStream_t s)
{
    k_sync_masters<T><<<dim3(64, b.ncases), 256, 0, s>>>(b.dcases, b.ncases);
    count_launch();
}

template <typename T> void launch_posdin(const Batch<T> &b, cudaStream_t s)
{
    k_posdin<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
template <typename T> void launch_conmassa(const Batch<T> &b, cudaStream_t s)
{
    k_conmassa<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
template <typename T> void launch_mms_error(const Batch<T> &b, cudaStream_t s)
{
    k_mms_error<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}
template <typename T> void launch_set_scalar(const Batch<T> &b, int slot, double v, cudaStream_t s)
{
    k_set_scalar<T><<<(b.ncases + 127) / 128, 128, 0, s>>>(b.dcases, b.ncases, slot, v); count_launch();
}

#define INST(T)                                                              \
    template void launch_visco<T>(const Batch<T> &, int, const double *, cudaStream_t); \
    template void launch_convdiff<T>(const Batch<T> &, int, cudaStream_t);  \
    template void launch_sponge<T>(const Batch<T> &, cudaStream_t);         \
    template void launch_complementos<T>(const Batch<T> &, cudaStream_t);   \
    template void launch_tempo<T>(const Batch<T> &, int, int, cudaStream_t);          \
    template void launch_posdin<T>(const Batch<T> &, cudaStream_t);         \
    template void launch_sync_masters<T>(const Batch<T> &, cudaStream_t);   \
    template void launch_conmassa<T>(const Batch<T> &, cudaStream_t);       \
    template void launch_mms_error<T>(const Batch<T> &, cudaStream_t);      \
    template void launch_set_scalar<T>(const Batch<T> &, int, double, cudaStream_t);
INST(double)
INST(float)

}  // namespace suli
