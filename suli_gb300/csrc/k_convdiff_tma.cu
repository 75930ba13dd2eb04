// k_convdiff_tma.cu -- convdiff (6_convdiff.f90:14-167, classico der = 3,
// 7_advectivo.f90:171-284), fused with complementos (11_diversos.f90:355-450),
// with its operands staged in shared memory by the Tensor Memory Accelerator.
//
// The kernel covers the interior positions, 2 <= i <= nx - 1, 2 <= j <=
// ny - 1, 2 <= k <= nz - 1, where all three faces exist and every boundary
// branch of the stencils takes its interior case; the boundary shell (i, j or
// k in {1, n, n + 1}) follows in a second launch, k_convdiff_shell, one
// thread per shell position reading global memory with the general stencils.
// Both run the per-face arithmetic of conv_faces.cuh.
//
// Work unit: a column of 32 x 8 positions (i, j) -- one per thread of a 32 x
// 8 block -- and CD_Z planes k (8, 16 or 32: the autotuner's choice); each
// thread forms Fu, Fv and Fw at its (i, j, k) for every k of the column.  The stencils reach two cells along every
// axis, so for each plane p the block stages, for each of the eight operand
// arrays (u, v, w, rho, mu, xmu, ymu, zmu), the box x in [i0 - 2, i0 + 38),
// y in [j0 - 2, j0 + 10) of plane p: one 40 x 12 x 1 cp.async.bulk.tensor
// load per array from a per-case tensor map of the array's padded box (x
// starts on a 16-byte boundary: i0 - 2 is a multiple of 32).  An interior
// thread reads every operand at a fixed offset from its own position in one
// of five plane slots.  Planes live in a ring of six slots; a plane is needed
// while the planes within two of it are computed, so plane k + 4 is loaded
// while plane k is computed.  Each slot has an mbarrier that the elected
// thread arms with the slot's transaction bytes; every wait is bounded, and a
// wait that gives up marks the case (S_TMAERR, reported as
// SULI_DEVICE_TIMEOUT) and ends the unit after the copies it issued have
// landed or their waits have run out (each wait gives up after a second).
#include "conv_faces.cuh"
#include "tma_util.cuh"

namespace suli {

constexpr int CD_X = 32, CD_Y = 8;              // unit: positions per thread block (x, y)
constexpr int CD_BX = CD_MAP_BOX_X, CD_BY = CD_MAP_BOX_Y;   // staged box of one array and plane
constexpr int CD_BOX = CD_BX * CD_BY;
constexpr int CD_NARR = 8;                       // u, v, w, rho, mu, xmu, ymu, zmu
constexpr int CD_RING = 6;                       // plane slots
constexpr int CD_SLOT = CD_NARR * CD_BOX;        // elements of one slot

// units of a case with kz planes a unit (kz = CD_PLANES[v], the tuner's choice)
__host__ __device__ __forceinline__ int cd_units(int nx, int ny, int nz, int kz)
{
    return ((nx - 2 + CD_X - 1) / CD_X) * ((ny - 2 + CD_Y - 1) / CD_Y) * ((nz - 2 + kz - 1) / kz);
}

template <typename T> constexpr size_t cd_smem() { return (size_t)CD_RING * CD_SLOT * sizeof(T) + 128; }

// operands from the staged planes (CHK: positions outside the staged box read
// global memory)
template <typename T, bool CHK>
struct StagedAcc {
    const CaseDev<T> &c;
    const T *S;
    int X0, Y0, kk;
    int p0, p1, p2, p3, p4;   // element offsets of the slots of planes kk-2 .. kk+2
    __device__ __forceinline__ T ld(int arr, const T *gsrc, int a, int b, int d) const
    {
        const int e = d - kk + 2;
        if (CHK) {
            if ((unsigned)(a - X0) >= (unsigned)CD_BX || (unsigned)(b - Y0) >= (unsigned)CD_BY || (unsigned)e > 4u)
                return gsrc[c.g.at(a, b, d)];
        }
        const int pb = e == 0 ? p0 : e == 1 ? p1 : e == 2 ? p2 : e == 3 ? p3 : p4;
        return S[pb + arr * CD_BOX + (a - X0) + CD_BX * (b - Y0)];
    }
    __device__ __forceinline__ T u(int a, int b, int d) const { return ld(0, c.u, a, b, d); }
    __device__ __forceinline__ T v(int a, int b, int d) const { return ld(1, c.v, a, b, d); }
    __device__ __forceinline__ T w(int a, int b, int d) const { return ld(2, c.w, a, b, d); }
    __device__ __forceinline__ T rho(int a, int b, int d) const { return ld(3, c.rho, a, b, d); }
    __device__ __forceinline__ T mu(int a, int b, int d) const { return ld(4, c.mu, a, b, d); }
    __device__ __forceinline__ T xmu(int a, int b, int d) const { return ld(5, c.xmu, a, b, d); }
    __device__ __forceinline__ T ymu(int a, int b, int d) const { return ld(6, c.ymu, a, b, d); }
    __device__ __forceinline__ T zmu(int a, int b, int d) const { return ld(7, c.zmu, a, b, d); }
};

// interior positions: every operand lies at a fixed offset from the
// thread's own position in the slots of planes k-2 .. k+2, so each load is
// one shared-memory access from one of five per-plane base pointers
template <typename T>
struct InteriorAcc {
    const T *P0, *P1, *P2, *P3, *P4;   // slots of planes k-2 .. k+2 at the thread's (i, j)
    int i, j, k;
    __device__ __forceinline__ T ld(int arr, int a, int b, int d) const
    {
        const int e = d - k + 2;
        const T *P = e == 0 ? P0 : e == 1 ? P1 : e == 2 ? P2 : e == 3 ? P3 : P4;
        return P[arr * CD_BOX + (a - i) + CD_BX * (b - j)];
    }
    __device__ __forceinline__ T u(int a, int b, int d) const { return ld(0, a, b, d); }
    __device__ __forceinline__ T v(int a, int b, int d) const { return ld(1, a, b, d); }
    __device__ __forceinline__ T w(int a, int b, int d) const { return ld(2, a, b, d); }
    __device__ __forceinline__ T rho(int a, int b, int d) const { return ld(3, a, b, d); }
    __device__ __forceinline__ T mu(int a, int b, int d) const { return ld(4, a, b, d); }
    __device__ __forceinline__ T xmu(int a, int b, int d) const { return ld(5, a, b, d); }
    __device__ __forceinline__ T ymu(int a, int b, int d) const { return ld(6, a, b, d); }
    __device__ __forceinline__ T zmu(int a, int b, int d) const { return ld(7, a, b, d); }
};

// an interior position: all three faces exist and every boundary branch of
// the stencils takes its interior case
template <typename T, bool CHK>
__device__ __forceinline__ void cd_interior_pos(const CaseDev<T> &c, const StagedAcc<T, CHK> &X, int i, int j, int k,
                                                int fuse)
{
    const int o = (i - X.X0) + CD_BX * (j - X.Y0);
    const InteriorAcc<T> Y{X.S + X.p0 + o, X.S + X.p1 + o, X.S + X.p2 + o, X.S + X.p3 + o, X.S + X.p4 + o, i, j, k};
    const long long q = c.g.at(i, j, k);
    T F = face_fu<T, InteriorAcc<T>, true>(c, Y, i, j, k);
    if (fuse) F = compl_fu<T>(c, F, i, j, k);
    c.Fu[q] = F;
    F = face_fv<T, InteriorAcc<T>, true>(c, Y, i, j, k);
    if (fuse) F = compl_fv<T>(c, F, i, j, k);
    c.Fv[q] = F;
    F = face_fw<T, InteriorAcc<T>, true>(c, Y, i, j, k);
    if (fuse) F = compl_fw<T>(c, F, Y.w(i, j, k), i, j, k);
    c.Fw[q] = F;
}

template <typename T, int CD_Z>
__global__ void __launch_bounds__(CD_X *CD_Y, sizeof(T) == 4 ? 2 : 1)
    k_convdiff_tma(const CaseDev<T> *__restrict__ cs, int ncases, const CUtensorMap *__restrict__ maps, int fuse, int v,
                   int shortfall)
{
    extern __shared__ unsigned char cd_dyn[];
    __shared__ __align__(8) uint64_t bar[CD_RING];
    T *S = reinterpret_cast<T *>(((uintptr_t)cd_dyn + 127) & ~(uintptr_t)127);
    // the case of this block: last case whose first unit is <= blockIdx.x
    int lo = 0, hi = ncases - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cs[mid].cd_begin[v] <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const CaseDev<T> &c = cs[lo];
    const int u = (int)blockIdx.x - c.cd_begin[v];
    const int nx = c.g.nx, ny = c.g.ny, nz = c.g.nz;
    const int ux = (nx - 2 + CD_X - 1) / CD_X, uy = (ny - 2 + CD_Y - 1) / CD_Y;
    const int ax = u % ux;
    const int i0 = 2 + ax * CD_X, j0 = 2 + ((u / ux) % uy) * CD_Y;
    const int k0 = 2 + (u / (ux * uy)) * CD_Z, k1 = min(nz - 1, k0 + CD_Z - 1);
    const int X0 = i0 - 2, Y0 = j0 - 2;   // X0 = 32 ax: a 16-byte boundary
    const CUtensorMap *tm = maps + (size_t)lo * CD_NARR;
    const int t = threadIdx.x + CD_X * threadIdx.y;
    const unsigned bytes = (unsigned)(CD_SLOT * sizeof(T));
    if (t == 0) {
        for (int s = 0; s < CD_RING; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        for (int a = 0; a < CD_NARR; ++a)
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(tm + a) : "memory");
    }
    __syncthreads();
    const int pl = k1 + 2;   // last plane any position of the unit reads
    // failure-path test hook (shortfall != 0): the unit's last plane is armed
    // with 16 bytes that no copy delivers, so its bounded wait runs out --
    // only while the case has no timeout recorded, so one launch pays the
    // wait and the later ones run normally
    const bool sf = shortfall != 0 && t == 0 && __ldcg(&c.sc[S_TMAERR]) == 0.0;
    auto slot = [](int p) { return (p + CD_RING) % CD_RING; };   // p >= -1
    auto issue = [&](int p) {
        const int s = slot(p);
        mbar_arm(&bar[s], bytes + (sf && p == pl ? 16u : 0u));
        T *dst = S + (size_t)s * CD_SLOT;
        for (int a = 0; a < CD_NARR; ++a) tma_load_3d(dst + a * CD_BOX, tm + a, X0, Y0, p, &bar[s]);
    };
    int issued = min(pl, k0 + 3);      // the same in every thread: thread 0 issues, all wait
    if (t == 0)
        for (int p = k0 - 2; p <= issued; ++p) issue(p);
    unsigned par = 0;          // bit s: parity of the next completion of slot s
    int waited = k0 - 3;       // planes up to this one have landed
    auto wait_to = [&](int last) {
        bool good = true;
        for (int p = waited + 1; p <= last; ++p) {
            const int s = slot(p);
            if (!mbar_wait(&bar[s], (par >> s) & 1u)) good = false;
            par ^= 1u << s;
        }
        waited = max(waited, last);
        return good;
    };
    // thread (tx, ty): position (i0 + tx, j0 + ty) of the interior range
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    const bool inside = i <= nx - 1 && j <= ny - 1;
    bool ok = __syncthreads_and(wait_to(min(k0 + 2, pl)));   // planes k0-2 .. k0+2
    for (int kk = k0; kk <= k1 && ok; ++kk) {
        const int p0 = slot(kk - 2) * CD_SLOT, p1 = slot(kk - 1) * CD_SLOT, p2 = slot(kk) * CD_SLOT,
                  p3 = slot(kk + 1) * CD_SLOT, p4 = slot(kk + 2) * CD_SLOT;
        if (inside) {
            const StagedAcc<T, false> X{c, S, X0, Y0, kk, p0, p1, p2, p3, p4};
            cd_interior_pos<T, false>(c, X, i, j, kk, fuse);
        }
        // the next plane's last input, then one barrier: every thread is done
        // with plane kk - 2, whose slot takes plane kk + 4
        const bool good = (kk < k1) ? wait_to(min(kk + 3, pl)) : true;
        ok = __syncthreads_and(good);
        if (ok && kk + 4 <= pl) {
            if (t == 0) {
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                issue(kk + 4);
            }
            issued = kk + 4;
        }
    }
    if (!ok) {
        // a copy did not land in time: mark the case, then wait (bounded) for
        // the copies this unit issued so that none lands after the block ends
        if (t == 0) c.sc[S_TMAERR] = 1.0;
        wait_to(issued);
    }
}

// The boundary shell as three slabs, each enumerated densely so that a warp's
// threads take consecutive positions: X = {1, nx, nx + 1} x [1, ny + 1] x
// [1, nz + 1], Y = [2, nx - 1] x {1, ny, ny + 1} x [1, nz + 1], Z = [2, nx - 1] x
// [2, ny - 1] x {1, nz, nz + 1}; the union is the complement of the interior.
__host__ __device__ __forceinline__ long long cd_shell_count(int nx, int ny, int nz)
{
    return 3LL * (ny + 1) * (nz + 1) + 3LL * (nx - 2) * (nz + 1) + 3LL * (nx - 2) * (ny - 2);
}

template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_convdiff_shell(const CaseDev<T> *__restrict__ cs, int ncases, int fuse,
                                                        long long total)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total) return;
    int lo = 0, hi = ncases - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cs[mid].cd_shell_begin <= q) lo = mid; else hi = mid - 1;
    }
    const CaseDev<T> &c = cs[lo];
    const int nx = c.g.nx, ny = c.g.ny, nz = c.g.nz;
    long long r = q - c.cd_shell_begin;
    int i, j, k;
    const long long nxs = 3LL * (ny + 1) * (nz + 1), nys = 3LL * (nx - 2) * (nz + 1);
    if (r < nxs) {                 // j fastest: neighbouring threads share the rows j +- 1, 2
        j = 1 + (int)(r % (ny + 1));
        r /= (ny + 1);
        const int e = (int)(r % 3);
        k = 1 + (int)(r / 3);
        i = e == 0 ? 1 : (e == 1 ? nx : nx + 1);
    } else if ((r -= nxs) < nys) {
        i = 2 + (int)(r % (nx - 2));
        r /= (nx - 2);
        const int e = (int)(r % 3);
        k = 1 + (int)(r / 3);
        j = e == 0 ? 1 : (e == 1 ? ny : ny + 1);
    } else {
        r -= nys;
        i = 2 + (int)(r % (nx - 2));
        r /= (nx - 2);
        j = 2 + (int)(r % (ny - 2));
        const int e = (int)(r / (ny - 2));
        k = e == 0 ? 1 : (e == 1 ? nz : nz + 1);
    }
    const GlobalAcc<T> X{c};
    const Geo &g = c.g;
    if (i <= nx + 1 && j <= ny && k <= nz) {
        T F = face_fu<T>(c, X, i, j, k);
        if (fuse) F = compl_fu<T>(c, F, i, j, k);
        c.Fu[g.at(i, j, k)] = F;
    }
    if (i <= nx && j <= ny + 1 && k <= nz) {
        T F = face_fv<T>(c, X, i, j, k);
        if (fuse) F = compl_fv<T>(c, F, i, j, k);
        c.Fv[g.at(i, j, k)] = F;
    }
    if (i <= nx && j <= ny && k <= nz + 1) {
        T F = face_fw<T>(c, X, i, j, k);
        if (fuse) F = compl_fw<T>(c, F, c.w[g.at(i, j, k)], i, j, k);
        c.Fw[g.at(i, j, k)] = F;
    }
}

long long convdiff_shell_positions(int nx, int ny, int nz) { return cd_shell_count(nx, ny, nz); }

template <typename T, int KZ> static void launch_tma_kz(const Batch<T> &b, int fuse, int v, cudaStream_t s)
{
    cudaFuncSetAttribute((const void *)k_convdiff_tma<T, KZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cd_smem<T>());
    k_convdiff_tma<T, KZ><<<b.total_cd_units[v], dim3(CD_X, CD_Y), cd_smem<T>(), s>>>(b.dcases, b.ncases, b.tmaps,
                                                                                      fuse, v, b.test_shortfall);
}

template <typename T> void launch_convdiff_tma(const Batch<T> &b, int fuse, cudaStream_t s)
{
    const int v = b.tune.cd_variant;
    if (v == 0) launch_tma_kz<T, 8>(b, fuse, 0, s);
    else if (v == 2) launch_tma_kz<T, 32>(b, fuse, 2, s);
    else launch_tma_kz<T, 16>(b, fuse, 1, s);
    count_launch();
    // the boundary shell (i, j or k at the domain's edges): the general stencils
    const long long n = b.total_cd_shell;
    k_convdiff_shell<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b.dcases, b.ncases, fuse, n);
    count_launch();
}

int convdiff_units(int nx, int ny, int nz, int variant) { return cd_units(nx, ny, nz, CD_PLANES[variant]); }

template void launch_convdiff_tma<float>(const Batch<float> &, int, cudaStream_t);
template void launch_convdiff_tma<double>(const Batch<double> &, int, cudaStream_t);

}  // namespace suli
