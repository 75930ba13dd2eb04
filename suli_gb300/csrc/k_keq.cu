// k_keq.cu -- the k-equation model of visco (m_turb = 2 LES, 3 DES;
// 5_viscosidade.f90:91-145), the explicit pressure force of the implicit
// pressure algorithm (exp_press, 11_diversos.f90:455-495) and the inflow
// waves (boundary_waves, 3_contorno.f90:1189-1319).
//
// k equation, per RK sub-stage tt = 1..ntt of visco's own loop (velocity,
// density and the strain sum p1 + p2 + p3 fixed over the loop; k_visco_mu
// stores the strain sum):
//   k_keq_nut     clamp of the previous sub-stage (ka < 0 -> 0, :131-139),
//                 nut = cmu sqrt(ka) delta (:100)
//   k_keq_rhs     Fka = -adv_esc(ka) + diffusion with ls_mu + nut rho over rho
//                 (convdiff_les, 6_convdiff.f90:171-205; adv_esc
//                 7_advectivo.f90:654-706) + nut 2 S^2 - des ka^1.5 / lcar (:115-124)
//   k_keq_update  tempo_esc (11_diversos.f90:300-351)
//   k_keq_bc x3   contorno_les (3_contorno.f90:666-790): y planes, z planes,
//                 x planes, each over the whole extent of the other indices,
//                 in the reference's order (edges take the later value)
// then k_keq_final: the last clamp, nut, mut = nut rho (:143-144), mu.
// The right-hand side and the update are separate launches because the
// update overwrites ka, which the right-hand side reads at the neighbours.
//
// exp_press: k_exp_press_faces forms px/py/pz from prdaux = prd1 + (prd1 +
// prd0), recomputed at each point with the same two roundings as the
// reference's prd0 = prd1 + prd0; prdaux = prd1 + prd0; then
// k_exp_press_acc stores prd0 += prd1 over the whole box.
#include "suli_kernels.cuh"

namespace suli {

#define AT(arr, i, j, k) (arr)[g.at((i), (j), (k))]

template <typename T, typename F>
__device__ __forceinline__ T icf_k(int f, int n, bool periodic, F get)
{
    if (f >= 2 && f <= n) return (get(f) + get(f - 1)) * T(0.5);
    if (periodic) return (get(1) + get(n)) * T(0.5);
    if (f == 1) return (get(2) + get(1)) * T(0.5);
    return (get(n) + get(n - 1)) * T(0.5);
}

// derivaxu2n/p etc. (8_derivadas.f90:75-300) along one axis of a haloed array
template <typename T, typename F>
__device__ __forceinline__ T u2n(int m, int dim, bool per, T rh, F a)
{
    if (m >= 2) return T(0.5) * (a(m - 2) - 4 * a(m - 1) + 3 * a(m)) * rh;
    if (!per) return T(0.5) * (a(m + 1) - a(m - 1)) * rh;
    return T(0.5) * (a(dim - 1) - 4 * a(dim) + 3 * a(m)) * rh;
}
template <typename T, typename F>
__device__ __forceinline__ T u2p(int m, int dim, bool per, T rh, F a)
{
    if (m <= dim - 1) return T(0.5) * (-a(m + 2) + 4 * a(m + 1) - 3 * a(m)) * rh;
    if (!per) return T(0.5) * (a(m + 1) - a(m - 1)) * rh;
    return T(0.5) * (-a(2) + 4 * a(1) - 3 * a(m)) * rh;
}

template <typename T>
__device__ __forceinline__ T upw_k(T vel, T dneg, T dpos)
{
    T a1 = vel > T(0.) ? vel : T(0.);
    T a2 = vel < T(0.) ? vel : T(0.);
    return a1 * dneg + a2 * dpos;
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_keq_nut(const CaseDev<T> *__restrict__ cs, int ncases, int clamp)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.m_turb < 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const long long q = g.at(i, j, k);
    T kv = c.ka[q];
    if (clamp && kv < T(0.)) {
        kv = T(0.);
        c.ka[q] = kv;
    }
    c.nut[q] = T(c.cmu) * sqrt(kv) * T(c.delta);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_keq_rhs(const CaseDev<T> *__restrict__ cs, int ncases, int tt)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.m_turb < 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (i > nx || j > ny || k > nz) return;
    const bool per = (c.ccx0 == 0);
    const long long q = g.at(i, j, k);
    const T *__restrict__ ka = c.ka;
    const T rx = T(c.idx), ry = T(c.idy), rz = T(c.idz);
    auto K = [&](int a, int b, int d) { return AT(ka, a, b, d); };
    // adv_esc: face velocities averaged to the centre, 2nd-order upwind
    const T uc = (AT(c.u, i, j, k) + AT(c.u, i + 1, j, k)) * T(0.5);
    const T vc = (AT(c.v, i, j, k) + AT(c.v, i, j + 1, k)) * T(0.5);
    const T wc = (AT(c.w, i, j, k) + AT(c.w, i, j, k + 1)) * T(0.5);
    const T adv = upw_k<T>(uc, u2n<T>(i, nx, per, rx, [&](int m) { return K(m, j, k); }),
                           u2p<T>(i, nx, per, rx, [&](int m) { return K(m, j, k); })) +
                  upw_k<T>(vc, u2n<T>(j, ny, false, ry, [&](int m) { return K(i, m, k); }),
                           u2p<T>(j, ny, false, ry, [&](int m) { return K(i, m, k); })) +
                  upw_k<T>(wc, u2n<T>(k, nz, false, rz, [&](int m) { return K(i, j, m); }),
                           u2p<T>(k, nz, false, rz, [&](int m) { return K(i, j, m); }));
    // diffusion: mu = ls_mu + nut rho interpolated to the faces (interp?_cf)
    auto mua = [&](int a, int b, int d) {
        const long long qq = g.at(a, b, d);
        return c.ls_mu[qq] + c.nut[qq] * c.rho[qq];
    };
    const T am1 = icf_k<T>(i + 1, nx, per, [&](int m) { return mua(m, j, k); });
    const T am0 = icf_k<T>(i, nx, per, [&](int m) { return mua(m, j, k); });
    const T bm1 = icf_k<T>(j + 1, ny, false, [&](int m) { return mua(i, m, k); });
    const T bm0 = icf_k<T>(j, ny, false, [&](int m) { return mua(i, m, k); });
    const T dm1 = icf_k<T>(k + 1, nz, false, [&](int m) { return mua(i, j, m); });
    const T dm0 = icf_k<T>(k, nz, false, [&](int m) { return mua(i, j, m); });
    const T kc = ka[q];
    T F = -adv + ((am1 * (K(i + 1, j, k) - kc) - am0 * (kc - K(i - 1, j, k))) * (rx * rx) +
                  (bm1 * (K(i, j + 1, k) - kc) - bm0 * (kc - K(i, j - 1, k))) * (ry * ry) +
                  (dm1 * (K(i, j, k + 1) - kc) - dm0 * (kc - K(i, j, k - 1))) * (rz * rz)) /
                     c.rho[q];
    // production and dissipation (:100-122): diss = ka^1.5 / lcar; DES limiter
    // max(1, ka^1.5 / (cdes delta diss)), whose 0/0 at ka = 0 gives 1 as the
    // reference's MAX does
    const T k15 = kc * sqrt(kc);
    const T diss = k15 / T(c.lcar);
    T des = T(1.);
    if (c.m_turb == 3) des = fmax(T(1.), k15 / (T(c.cdes) * T(c.delta) * diss));
    const T sm = c.sij[q];
    F = F + c.nut[q] * T(2.) * sm * sm - des * diss;
    T *out = (tt == 1) ? c.fk0 : (tt == 2) ? c.fk1 : c.fka;
    out[q] = F;
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_keq_update(const CaseDev<T> *__restrict__ cs, int ncases, int tt, double dt)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.m_turb < 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const long long q = g.at(i, j, k);
    const T d = T(dt);
    if (tt == 1) {
        const T e = c.ka[q];
        c.ka0[q] = e;
        c.ka[q] = e + d * c.fk0[q];
    } else if (tt == 2) {
        const T aux1 = T(2.) * d;
        c.ka[q] = c.ka0[q] - d * c.fk0[q] + aux1 * c.fk1[q];
    } else {
        const T aux1 = d / T(6.);
        c.ka[q] = c.ka0[q] + aux1 * (c.fk0[q] + T(4.) * c.fk1[q] + c.fka[q]);
    }
}

// contorno_les, one phase (0: y planes, 1: z planes, 2: x planes); grid x
// strides the plane, grid y = case
template <typename T>
__global__ void k_keq_bc(const CaseDev<T> *__restrict__ cs, int ncases, int phase)
{
    const CaseDev<T> &c = cs[blockIdx.y];
    if (c.m_turb < 2) return;
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    T *__restrict__ ka = c.ka;
    long long n;
    if (phase == 0) n = (long long)(nx + 2) * (nz + 2);
    else if (phase == 1) n = (long long)(nx + 2) * (ny + 2);
    else n = (long long)(ny + 2) * (nz + 2);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        if (phase == 0) {
            const int i = (int)(t % (nx + 2)), k = (int)(t / (nx + 2));
            if (c.ccy0 == 0 && c.ccyf == 0) {
                AT(ka, i, ny + 1, k) = AT(ka, i, 1, k);
                AT(ka, i, 0, k) = AT(ka, i, ny, k);
            }
            if (c.ccy0 == 1) AT(ka, i, 0, k) = AT(ka, i, 1, k);
            if (c.ccyf == 1) AT(ka, i, ny + 1, k) = AT(ka, i, ny, k);
            if (c.ccy0 == 2) AT(ka, i, 0, k) = -AT(ka, i, 1, k);
            if (c.ccyf == 2) AT(ka, i, ny + 1, k) = -AT(ka, i, ny, k);
        } else if (phase == 1) {
            const int i = (int)(t % (nx + 2)), j = (int)(t / (nx + 2));
            if (c.ccz0 == 1) AT(ka, i, j, 0) = AT(ka, i, j, 1);
            if (c.cczf == 1) AT(ka, i, j, nz + 1) = AT(ka, i, j, nz);
            if (c.ccz0 == 2 || c.ccz0 == 4) AT(ka, i, j, 0) = -AT(ka, i, j, 1);
        } else {
            const int j = (int)(t % (ny + 2)), k = (int)(t / (ny + 2));
            if (c.ccx0 == 0 && c.ccxf == 0) {
                AT(ka, nx + 1, j, k) = AT(ka, 1, j, k);
                AT(ka, 0, j, k) = AT(ka, nx, j, k);
            }
            if (c.ccx0 == 1) AT(ka, 0, j, k) = AT(ka, 1, j, k);
            if (c.ccxf == 1 || c.ccxf == 4) AT(ka, nx + 1, j, k) = AT(ka, nx, j, k);
            if (c.ccx0 == 2) AT(ka, 0, j, k) = -AT(ka, 1, j, k);
            if (c.ccxf == 2) AT(ka, nx + 1, j, k) = -AT(ka, nx, j, k);
            if (c.ccx0 == 3 && j >= 1 && j <= ny && k >= 1 && k <= nz)
                AT(ka, 0, j, k) = T(c.iturb * c.iturb * c.uinicial * c.uinicial * 1.5);
            if (c.ccxf == 3) AT(ka, nx + 1, j, k) = AT(ka, nx, j, k);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_keq_final(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.m_turb < 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    const long long q = g.at(i, j, k);
    T kv = c.ka[q];
    if (kv < T(0.)) {
        kv = T(0.);
        c.ka[q] = kv;
    }
    const T nut = T(c.cmu) * sqrt(kv) * T(c.delta);
    const T mut = nut * c.rho[q];
    c.nut[q] = nut;
    c.mut[q] = mut;
    c.mu[q] = c.ls_mu[q] + mut;
}

// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_exp_press_faces(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (!c.ipa) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool per = (c.ccx0 == 0);
    auto pa = [&](int a, int b, int d) {
        const long long qq = g.at(a, b, d);
        const T p1 = c.prd1[qq];
        return p1 + (p1 + c.prd0[qq]);
    };
    auto rho = [&](int a, int b, int d) { return c.rho[g.at(a, b, d)]; };
    const long long q = g.at(i, j, k);
    const T pc = (i <= nx + 1 && j <= ny + 1 && k <= nz + 1) ? pa(i, j, k) : T(0.);
    if (i <= nx + 1 && j <= ny && k <= nz)
        c.px[q] = -(pc - pa(i - 1, j, k)) / T(c.dx) / icf_k<T>(i, nx, per, [&](int m) { return rho(m, j, k); });
    if (i <= nx && j <= ny + 1 && k <= nz)
        c.py[q] = -(pc - pa(i, j - 1, k)) / T(c.dy) / icf_k<T>(j, ny, false, [&](int m) { return rho(i, m, k); });
    if (i <= nx && j <= ny && k <= nz + 1)
        c.pz[q] = -(pc - pa(i, j, k - 1)) / T(c.dz) / icf_k<T>(k, nz, false, [&](int m) { return rho(i, j, m); });
}

// prd0 = prd1 + prd0 on the whole box (0:nx+1, 0:ny+1, 0:nz+1); grid x
// strides the case's box, grid y = case
template <typename T>
__global__ void k_exp_press_acc(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[blockIdx.y];
    if (!c.ipa) return;
    const Geo &g = c.g;
    const long long n = g.total;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        c.prd0[q] = c.prd1[q] + c.prd0[q];
}

// ---------------------------------------------------------------------------
// boundary_waves (3_contorno.f90:1189-1319) at time t: the wave on the columns
// i = 0, 1 over j = 0..ny+1, k = 0..nz+1 (kp(k) = (k - 0.5) dz), in FP64;
// ls(1, :, :) takes the surface (and its FP64 master in the mixed form),
// bxx0 / bxz0 the i = 0 velocities, bxx1 the i = 1 u.  Grid: x strides the
// plane, y = case.
template <typename T>
__global__ void k_waves(const CaseDev<T> *__restrict__ cs, int ncases, double t, int tdev)
{
    if (tdev) t = cs[0].sc[S_TIME];
    const CaseDev<T> &c = cs[blockIdx.y];
    if (c.wave_t <= 0) return;
    const Geo &g = c.g;
    const int ny = g.ny, nz = g.nz;
    const long long pl = ny + 3;
    const double dx = c.dx, dz = c.dz, a_w = c.a_w, f_w = c.f_w, n_w = c.n_w, h0 = c.h0_f;
    const long long n = (long long)(ny + 2) * (nz + 2);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(q % (ny + 2)), k = (int)(q / (ny + 2));
        const double kp = (k - 0.5) * dz;
        for (int i = 0; i <= 1; ++i) {
            const double aux2 = n_w * dx * (i - 0.5) - f_w * t, aux3 = n_w * dx * (i - 1.) - f_w * t;
            double h_f, u1 = 0., w1 = 0.;
            if (c.wave_t == 1) {
                h_f = h0 + a_w * cos(aux2);
                if (h_f - kp >= 0.) {
                    u1 = a_w * f_w * cosh(n_w * kp) / sinh(n_w * h0) * cos(aux3);
                    w1 = a_w * f_w * sinh(n_w * (kp - 0.5 * dz)) / sinh(n_w * h0) * sin(aux2);
                }
            } else if (c.wave_t == 2) {
                const double aux1 = tanh(n_w * h0);
                h_f = h0 + a_w * cos(aux2) + n_w * a_w * a_w * (3. - aux1 * aux1) / (4. * aux1 * aux1 * aux1) * cos(2. * aux2);
                if (h_f - kp >= 0.) {
                    const double s4 = pow(sinh(n_w * h0), 4.);
                    u1 = a_w * f_w * cosh(n_w * kp) / sinh(n_w * h0) * cos(aux3) +
                         3. / 4. * a_w * a_w * f_w * n_w * cosh(2. * n_w * kp) / s4 * cos(2. * aux3);
                    w1 = a_w * f_w * sinh(n_w * (kp - 0.5 * dz)) / sinh(n_w * h0) * sin(aux2) +
                         3. / 4. * a_w * a_w * f_w * n_w * sinh(2. * n_w * (kp - 0.5 * dz)) / s4 * sin(2. * aux3);
                }
            } else {
                const double aux4 = n_w * kp, aux5 = n_w * (kp - 0.5 * dz);
                h_f = h0 + c.aeta[0] * cos(aux2) + c.aeta[1] * cos(2. * aux2) + c.aeta[2] * cos(3. * aux2) +
                      c.aeta[3] * cos(4. * aux2) + c.aeta[4] * cos(5. * aux2);
                if (h_f - kp >= 0.) {
                    u1 = c.avel[0] * cosh(aux4) * cos(aux3) + c.avel[1] * cosh(2. * aux4) * cos(2. * aux3) +
                         c.avel[2] * cosh(3. * aux4) * cos(3. * aux3) + c.avel[3] * cosh(4. * aux4) * cos(4. * aux3) +
                         c.avel[4] * cosh(5. * aux4) * cos(5. * aux3);
                    w1 = c.avel[0] * sinh(aux5) * sin(aux2) + c.avel[1] * sinh(2. * aux5) * sin(2. * aux2) +
                         c.avel[2] * sinh(3. * aux5) * sin(3. * aux2) + c.avel[3] * sinh(4. * aux5) * sin(4. * aux2) +
                         c.avel[4] * sinh(5. * aux5) * sin(5. * aux2);
                }
            }
            if (i == 1 && j >= 1 && j <= ny && k >= 1 && k <= nz) {
                const long long qq = g.at(1, j, k);
                c.ls[qq] = T(h_f - kp);
                if (c.ls64) c.ls64[qq] = h_f - kp;
            }
            if (i == 0) {
                c.bxx0[j + pl * k] = T(u1);
                c.bxz0[j + pl * k] = T(w1);
            } else {
                c.bxx1[j + pl * k] = T(u1);
            }
        }
    }
}

// ---------------------------------------------------------------------------
static int plane_blocks(int max_plane)
{
    int nb = (max_plane + 255) / 256;
    return nb < 1 ? 1 : (nb > 1024 ? 1024 : nb);
}

template <typename T> void launch_contorno_les(const Batch<T> &b, cudaStream_t s)
{
    dim3 grid(plane_blocks(b.max_plane), b.ncases);
    for (int ph = 0; ph < 3; ++ph) {
        k_keq_bc<T><<<grid, 256, 0, s>>>(b.dcases, b.ncases, ph); count_launch();
    }
}

template <typename T> void launch_keq(const Batch<T> &b, int ntt, const double *a_dt, cudaStream_t s)
{
    for (int tt = 1; tt <= ntt; ++tt) {
        k_keq_nut<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, tt > 1 ? 1 : 0); count_launch();
        k_keq_rhs<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, tt); count_launch();
        k_keq_update<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, tt, a_dt[tt - 1]); count_launch();
        launch_contorno_les<T>(b, s);
    }
    k_keq_final<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
}

template <typename T> void launch_exp_press(const Batch<T> &b, cudaStream_t s)
{
    k_exp_press_faces<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases); count_launch();
    dim3 grid(1024, b.ncases);
    k_exp_press_acc<T><<<grid, 256, 0, s>>>(b.dcases, b.ncases); count_launch();
}

template <typename T> void launch_waves(const Batch<T> &b, double t, cudaStream_t s, int tdev)
{
    dim3 grid(plane_blocks(b.max_plane), b.ncases);
    k_waves<T><<<grid, 256, 0, s>>>(b.dcases, b.ncases, t, tdev); count_launch();
}

template void launch_waves<float>(const Batch<float> &, double, cudaStream_t, int);
template void launch_waves<double>(const Batch<double> &, double, cudaStream_t, int);
template void launch_contorno_les<float>(const Batch<float> &, cudaStream_t);
template void launch_contorno_les<double>(const Batch<double> &, cudaStream_t);
template void launch_keq<float>(const Batch<float> &, int, const double *, cudaStream_t);
template void launch_keq<double>(const Batch<double> &, int, const double *, cudaStream_t);
template void launch_exp_press<float>(const Batch<float> &, cudaStream_t);
template void launch_exp_press<double>(const Batch<double> &, cudaStream_t);

}  // namespace suli
