// k_ibm.cu -- image-point immersed boundary (ibm_t = 2), 15_ibm.f90.
//
//   k_ibm_posicoes    integer masks id_ibm* (15_ibm.f90:9-131): a solid point
//                     (obs > 0) within two points of a sign change along any
//                     axis; a pure per-point function, bit-exact
//   k_ibm_image       ibm_images (15_ibm.f90:134-318) pass 1: for every
//                     id = 1 point, two image points along the outward normal
//                     (normal from mod_ls1 of the obstacle level set, computed
//                     here on the fly with the same WENO derivatives),
//                     inverse-distance interpolation over the 8 surrounding
//                     points that are not id = 1, Auguste's quadratic
//                     extrapolation; the result goes to scratch
//   k_ibm_apply       pass 2: writes u = 2 v_sol - image (velocities) or
//                     ls = image (level set) and zeroes the solid interior
//   k_lsv_fill        fantasmas_cf (8_derivadas.f90:625-671): ls with ghosts
//
// The reference sweeps in place; its images never read a point the same
// sweep modifies with non-zero weight (modified id = 1 points carry weight
// 0, and zeroed interior points lie more than two cells inside the
// obstacle, beyond every image stencil), so the two-pass form gives the
// same values.  Indices of the image cells are formed with explicitly
// rounded FP64 operations so they agree with the oracle bit for bit.
#include "suli_kernels.cuh"

namespace suli {

#define AT(arr, i, j, k) (arr)[g.at((i), (j), (k))]

// WENO5 pieces shared with k_levelset.cu (re-declared here: kernels of one TU)
template <typename T>
__device__ __forceinline__ T iweno5(T v0, T v1, T v2, T v3, T v4)
{
    const T aux1 = T(13. / 12.), aux2 = T(1. / 4.), aux3 = T(1. / 6.), aux6 = T(0.00000001);
    T a, b;
    a = v0 - 2 * v1 + v2;
    b = v0 - 4 * v1 + 3 * v2;
    T is1 = aux1 * a * a + aux2 * b * b;
    a = v1 - 2 * v2 + v3;
    b = v1 - v3;
    T is2 = aux1 * a * a + aux2 * b * b;
    a = v2 - 2 * v3 + v4;
    b = 3 * v2 - 4 * v3 + v4;
    T is3 = aux1 * a * a + aux2 * b * b;
    T al1 = T(0.1) / ((aux6 + is1) * (aux6 + is1));
    T al2 = T(0.6) / ((aux6 + is2) * (aux6 + is2));
    T al3 = T(0.3) / ((aux6 + is3) * (aux6 + is3));
    T s = al1 + al2 + al3;
    T om1 = al1 / s, om2 = al2 / s, om3 = al3 / s;
    return aux3 * (om1 * (2 * v0 - 7 * v1 + 11 * v2) + om2 * (-v1 + 5 * v2 + 2 * v3) +
                   om3 * (2 * v2 + 5 * v3 - v4));
}

template <typename T>
__device__ void iline(const T *a, long long base, long long st, int i, int n, int ihs, T (&L)[7])
{
    for (int t = 0; t < 7; ++t) {
        int m = i - 3 + t;
        if (ihs == 0) {
            if (m < 1) m += n - 1;
            else if (m > n) m -= n - 1;
            L[t] = a[base + (long long)m * st];
        } else if (m >= 1 && m <= n) {
            L[t] = a[base + (long long)m * st];
        }
    }
    if (ihs != 0) {
        const T c11 = T(1. / 11.);
        if (i - 3 < 1) {
            T p1 = a[base + st], p2 = a[base + 2 * st], p3 = a[base + 3 * st];
            T g0 = c11 * (T(18.) * p1 - T(9.) * p2 + T(2.) * p3);
            T gm1 = c11 * (T(18.) * g0 - T(9.) * p1 + T(2.) * p2);
            T gm2 = c11 * (T(18.) * gm1 - T(9.) * g0 + T(2.) * p1);
            for (int t = 0; t < 7; ++t) {
                int m = i - 3 + t;
                if (m == 0) L[t] = g0;
                else if (m == -1) L[t] = gm1;
                else if (m == -2) L[t] = gm2;
            }
        }
        if (i + 3 > n) {
            T pn = a[base + (long long)n * st], pn1 = a[base + (long long)(n - 1) * st],
              pn2 = a[base + (long long)(n - 2) * st];
            T g1 = c11 * (T(18.) * pn - T(9.) * pn1 + T(2.) * pn2);
            T g2 = c11 * (T(18.) * g1 - T(9.) * pn + T(2.) * pn1);
            T g3 = c11 * (T(18.) * g2 - T(9.) * g1 + T(2.) * pn);
            for (int t = 0; t < 7; ++t) {
                int m = i - 3 + t;
                if (m == n + 1) L[t] = g1;
                else if (m == n + 2) L[t] = g2;
                else if (m == n + 3) L[t] = g3;
            }
        }
    }
}

// the larger-magnitude WENO derivative along one axis (mod_ls1, 14_level_set.f90:611-633)
template <typename T>
__device__ __forceinline__ T big_deriv(const T *a, long long base, long long st, int i, int n, int ihs, T h)
{
    T L[7];
    iline<T>(a, base, st, i, n, ihs, L);
    T D[6];
    for (int t = 0; t < 6; ++t) D[t] = (L[t + 1] - L[t]) / h;
    T dp = iweno5<T>(D[5], D[4], D[3], D[2], D[1]);
    T dn = iweno5<T>(D[0], D[1], D[2], D[3], D[4]);
    return (fabs(dp) > fabs(dn)) ? dp : dn;
}

// unit normal of the obstacle level set at a point (mod_ls1, :636-652)
template <typename T>
__device__ void obs_normal(const CaseDev<T> &c, const T *o, int i, int j, int k, int n0, int n1, int n2, double &nx,
                           double &ny, double &nz)
{
    const Geo &g = c.g;
    T a = big_deriv<T>(o, g.at(0, j, k), 1, i, n0, c.ccx0 == 0 ? 0 : 2, T(c.dx));
    T b = big_deriv<T>(o, g.at(i, 0, k), g.sx, j, n1, c.ccy0 == 0 ? 0 : 2, T(c.dy));
    T cc = big_deriv<T>(o, g.at(i, j, 0), g.sxy, k, n2, 2, T(c.dz));
    T m = sqrt(a * a + b * b + cc * cc);
    if (m == T(0)) { nx = ny = nz = 0.0; return; }
    nx = (double)(a / m); ny = (double)(b / m); nz = (double)(cc / m);
}

// target: 1 = u (x faces), 2 = v (y faces), 3 = w (z faces), 4 = level set
template <typename T>
struct IbmTarget {
    const T *obs;
    int *id;
    T *a1;
    int n0, n1, n2;            // extent of obs/id
    int lo0, hi0, lo1, hi1, lo2, hi2;  // index range of a1
    double ox, oy, oz;         // x(i) = (i - ox) dx
};

template <typename T>
__device__ __forceinline__ IbmTarget<T> ibm_target(const CaseDev<T> &c, int target)
{
    IbmTarget<T> t;
    const int nx = c.g.nx, ny = c.g.ny, nz = c.g.nz;
    t.n0 = nx; t.n1 = ny; t.n2 = nz;
    t.lo0 = t.lo1 = t.lo2 = 0;
    t.hi0 = nx + 1; t.hi1 = ny + 1; t.hi2 = nz + 1;
    t.ox = t.oy = t.oz = 0.5;
    if (target == 1) { t.obs = c.obs_lsx; t.id = c.id_ibmx; t.a1 = c.u; t.n0 = nx + 1; t.hi0 = nx + 2; t.ox = 1.0; }
    else if (target == 2) { t.obs = c.obs_lsy; t.id = c.id_ibmy; t.a1 = c.v; t.n1 = ny + 1; t.hi1 = ny + 2; t.oy = 1.0; }
    else if (target == 3) { t.obs = c.obs_lsz; t.id = c.id_ibmz; t.a1 = c.w; t.n2 = nz + 1; t.hi2 = nz + 2; t.oz = 1.0; }
    else { t.obs = c.obs_lss; t.id = c.id_ibm; t.a1 = c.lsb; }
    return t;
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_ibm_posicoes(const CaseDev<T> *__restrict__ cs, int ncases, int target)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.ibm_t != 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    IbmTarget<T> t = ibm_target(c, target);
    if (i > t.n0 || j > t.n1 || k > t.n2) return;
    const T *o = t.obs;
    T v = AT(o, i, j, k);
    int id = 0;
    if (v > T(0)) {
        if (i <= t.n0 - 2 && (v * AT(o, i + 1, j, k) < T(0.) || v * AT(o, i + 2, j, k) < T(0.))) id = 1;
        if (i >= 3 && (v * AT(o, i - 1, j, k) < T(0.) || v * AT(o, i - 2, j, k) < T(0.))) id = 1;
        if (j <= t.n1 - 2 && (v * AT(o, i, j + 1, k) < T(0.) || v * AT(o, i, j + 2, k) < T(0.))) id = 1;
        if (j >= 3 && (v * AT(o, i, j - 1, k) < T(0.) || v * AT(o, i, j - 2, k) < T(0.))) id = 1;
        if (k <= t.n2 - 2 && (v * AT(o, i, j, k + 1) < T(0.) || v * AT(o, i, j, k + 2) < T(0.))) id = 1;
        if (k >= 3 && (v * AT(o, i, j, k - 1) < T(0.) || v * AT(o, i, j, k - 2) < T(0.))) id = 1;
    }
    AT(t.id, i, j, k) = id;
}

__device__ __forceinline__ int clampi_(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_ibm_image(const CaseDev<T> *__restrict__ cs, int ncases, int target,
                                                        int der_t)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.ibm_t != 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    IbmTarget<T> t = ibm_target(c, target);
    if (i > t.n0 || j > t.n1 || k > t.n2) return;
    if (AT(t.id, i, j, k) != 1) return;
    const double dx = c.dx, dy = c.dy, dz = c.dz, deltai = c.deltai;
    const double er = deltai * 0.01, v_sol = 0.0;
    const double ob = (double)AT(t.obs, i, j, k);
    double image;
    if (ob < er) {
        image = (double)AT(t.a1, i, j, k);
    } else {
        double nxv, nyv, nzv, dummy0, dummy1;
        obs_normal<T>(c, t.obs, i, j, k, t.n0, t.n1, t.n2, nxv, nyv, nzv);
        if (k == 1 && t.n2 >= 2) obs_normal<T>(c, t.obs, i, j, k + 1, t.n0, t.n1, t.n2, dummy0, dummy1, nzv);
        // a component below the round-off of the obstacle level set is an
        // exact zero (z of an obstacle extruded along z); its sign would pick
        // the image cell through floor().  FP64 obstacle: 1e-9.  The mixed
        // form's FP32 obstacle, reinitialised in FP32 (the WENO end
        // extrapolation multiplies by a rounded 1/11), carries ~1e-6 of such
        // round-off near the bed: 1e-4 there
        const double zr = (sizeof(T) == 4) ? 1e-4 : 1e-9;
        nxv = fabs(nxv) < zr ? 0.0 : nxv;
        nyv = fabs(nyv) < zr ? 0.0 : nyv;
        nzv = fabs(nzv) < zr ? 0.0 : nzv;
        auto XC = [&](int a) { return __dmul_rn((double)a - t.ox, dx); };
        auto YC = [&](int a) { return __dmul_rn((double)a - t.oy, dy); };
        auto ZC = [&](int a) { return __dmul_rn((double)a - t.oz, dz); };
        double imp[2];
        for (int l = 1; l <= 2; ++l) {
            double xl = __dsub_rn(XC(i), __dmul_rn(__dadd_rn(__dmul_rn((double)l, dx), ob), nxv));
            double yl = __dsub_rn(YC(j), __dmul_rn(__dadd_rn(__dmul_rn((double)l, dy), ob), nyv));
            double zl = __dsub_rn(ZC(k), __dmul_rn(__dadd_rn(__dmul_rn((double)l, dz), ob), nzv));
            int ii = (int)floor(__ddiv_rn(__dsub_rn(xl, XC(i)), dx)) + i;
            int jj = (int)floor(__ddiv_rn(__dsub_rn(yl, YC(j)), dy)) + j;
            int kk = (int)floor(__ddiv_rn(__dsub_rn(zl, ZC(k)), dz)) + k;
            const int oi[8] = {0, 1, 0, 0, 1, 1, 0, 1}, oj[8] = {0, 0, 1, 0, 1, 0, 1, 1}, ok[8] = {0, 0, 0, 1, 0, 1, 1, 1};
            double lint[8], sl = 0.0, sv = 0.0;
            for (int q = 0; q < 8; ++q) {
                int I = ii + oi[q], J = jj + oj[q], K = kk + ok[q];
                double ddx = __dsub_rn(xl, XC(I)), ddy = __dsub_rn(yl, YC(J)), ddz = __dsub_rn(zl, ZC(K));
                int idv = (I < 1 || I > t.n0 || J < 1 || J > t.n1 || K < 1 || K > t.n2) ? 0 : AT(t.id, I, J, K);
                double d2 = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
                lint[q] = __dmul_rn(__ddiv_rn(1.0, __dsqrt_rn(d2)), (double)(1 - idv));
            }
            for (int q = 0; q < 8; ++q) sl = __dadd_rn(sl, lint[q]);
            for (int q = 0; q < 8; ++q) {
                int I = clampi_(ii + oi[q], t.lo0, t.hi0), J = clampi_(jj + oj[q], t.lo1, t.hi1),
                    K = clampi_(kk + ok[q], t.lo2, t.hi2);
                sv = __dadd_rn(sv, __dmul_rn(lint[q], (double)AT(t.a1, I, J, K)));
            }
            imp[l - 1] = (sl == 0.0) ? 0.0 : __ddiv_rn(sv, sl);
        }
        double li1 = __ddiv_rn(__dmul_rn(__ddiv_rn(__dsub_rn(2. * deltai, ob), deltai), 2. * ob), __dadd_rn(deltai, ob));
        double li2 = __ddiv_rn(__dmul_rn(__ddiv_rn(__dsub_rn(ob, deltai), deltai), 2. * ob), __dadd_rn(2. * deltai, ob));
        double lg = __ddiv_rn(__dmul_rn(__ddiv_rn(__dsub_rn(ob, deltai), __dadd_rn(ob, deltai)), __dsub_rn(ob, 2. * deltai)),
                              __dadd_rn(ob, 2. * deltai));
        double num;
        if (der_t == 1) num = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(2., lg), v_sol), __dmul_rn(li1, imp[0])), __dmul_rn(li2, imp[1]));
        else num = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(2., lg), imp[0]), __dmul_rn(li1, imp[0])), __dmul_rn(li2, imp[1]));
        image = __ddiv_rn(num, __dadd_rn(1., lg));
    }
    AT(c.mp, i, j, k) = T(image);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_ibm_apply(const CaseDev<T> *__restrict__ cs, int ncases, int target,
                                                        int der_t)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.ibm_t != 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    IbmTarget<T> t = ibm_target(c, target);
    if (i > t.n0 || j > t.n1 || k > t.n2) return;
    int id = AT(t.id, i, j, k);
    if (id == 1) {
        T im = AT(c.mp, i, j, k);
        AT(t.a1, i, j, k) = (der_t == 1) ? T(2.0 * 0.0) - im : im;
    } else if (der_t == 1 && AT(t.obs, i, j, k) > T(0.)) {
        AT(t.a1, i, j, k) = T(0.);
    }
}

// fantasmas_cf of ls into lsb (0:nx+1, 0:ny+1, 0:nz+1): y and z ghosts copy
// the adjacent interior value, edges not covered by those loops are 0 (as the
// zero-filled array of the oracle), then the x ghosts copy or wrap.
template <typename T>
__global__ void k_lsv_fill(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[blockIdx.y];
    if (c.ibm_t != 2) return;
    const Geo &g = c.g;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const long long n = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    const bool per = (c.ccx0 == 0);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % (nx + 2));
        long long r = t / (nx + 2);
        int j = (int)(r % (ny + 2)), k = (int)(r / (ny + 2));
        int im = i;
        if (i == 0) im = per ? nx : 1;
        else if (i == nx + 1) im = per ? 1 : nx;
        bool jin = (j >= 1 && j <= ny), kin = (k >= 1 && k <= nz);
        T v;
        if (jin && kin) v = AT(c.ls, im, j, k);
        else if (!jin && kin) v = AT(c.ls, im, j < 1 ? 1 : ny, k);
        else if (jin && !kin) v = AT(c.ls, im, j, k < 1 ? 1 : nz);
        else v = T(0.);
        AT(c.lsb, i, j, k) = v;
    }
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_lsv_back(const CaseDev<T> *__restrict__ cs, int ncases)
{
    const CaseDev<T> &c = cs[find_case(cs, ncases)];
    if (c.ibm_t != 2) return;
    int i, j, k;
    tile_ijk(c, i, j, k);
    const Geo &g = c.g;
    if (i > g.nx || j > g.ny || k > g.nz) return;
    AT(c.ls, i, j, k) = AT(c.lsb, i, j, k);
}

// ---- launchers -----------------------------------------------------------------
template <typename T> void launch_ibm_posicoes(const Batch<T> &b, cudaStream_t s)
{
    for (int t = 1; t <= 4; ++t) {
        k_ibm_posicoes<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, t);
        count_launch();
    }
}
template <typename T> void launch_ibm_velocity(const Batch<T> &b, cudaStream_t s)
{
    // u, v, w in turn, as 3_contorno.f90:87-89 (each reads only its own array)
    for (int t = 1; t <= 3; ++t) {
        k_ibm_image<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, t, 1);
        k_ibm_apply<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, t, 1);
        count_launch(2);
    }
}
template <typename T> void launch_ibm_levelset(const Batch<T> &b, cudaStream_t s)
{
    int nb = (b.max_plane + 255) / 256;
    nb = nb < 1 ? 1 : (nb > 2048 ? 2048 : nb);
    k_lsv_fill<T><<<dim3(nb, b.ncases), 256, 0, s>>>(b.dcases, b.ncases);
    k_ibm_image<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 4, 2);
    k_ibm_apply<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases, 4, 2);
    k_lsv_back<T><<<b.total_tiles, b.block(), 0, s>>>(b.dcases, b.ncases);
    count_launch(4);
}

template void launch_ibm_posicoes<double>(const Batch<double> &, cudaStream_t);
template void launch_ibm_velocity<double>(const Batch<double> &, cudaStream_t);
template void launch_ibm_levelset<double>(const Batch<double> &, cudaStream_t);
template void launch_ibm_posicoes<float>(const Batch<float> &, cudaStream_t);
template void launch_ibm_velocity<float>(const Batch<float> &, cudaStream_t);
template void launch_ibm_levelset<float>(const Batch<float> &, cudaStream_t);

}  // namespace suli
