// suli_api.cu -- the C ABI of include/suli_gpu.h.
//
// A handle owns a batch of device-resident cases (one case for the Fortran
// drop-in, many for an ensemble), a stream, the per-case scalar table and
// the reduction scratch.  Each entry point enqueues the kernels of one
// reference subroutine for every case of the batch; the only host reads are
// the loop-control flags of the CG (once per chunk of iterations), of the
// volume-correction loop (once per level_set) and explicit diagnostics.
#include "../../include/suli_gpu.h"
#include "suli_kernels.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace suli;

namespace suli {
std::atomic<unsigned long long> g_launches{0};
}

static thread_local std::string g_err;

static int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

#define CK(call)                                                                                \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(e_ == cudaErrorMemoryAllocation ? SULI_OUT_OF_MEMORY : SULI_CUDA_ERROR, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

#define CKL()                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = cudaGetLastError();                                                    \
        if (e_ != cudaSuccess) return fail(SULI_CUDA_ERROR, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
    } while (0)

extern "C" void suli_default_params(suli_params *p)
{
    std::memset(p, 0, sizeof(*p));
    p->t_tempo = 2;
    p->der = 3;
    p->adv_type = 1;
    p->t_press = 1;
    p->ccx0 = p->ccxf = p->ccy0 = p->ccyf = p->ccz0 = p->cczf = 1;
    p->gz = 9.80665;
    p->csmag = 0.13;
    p->alpha1 = 1.5;
    p->rho_f1 = 1.204;
    p->mu_f1 = 0.000018253;
    p->rho_f2 = 998.0;
    p->mu_f2 = 0.00100798;
    p->omp_t = 1;
    p->reinit_max_iter = 3;
    p->cg_max_iter = 10000;
    p->cg_tol_mode = SULI_CG_TOL_ABS;
    p->cg_tol = 1e-4;
    p->precision = SULI_PREC_FP64;
    p->vol_loop_max = 1000;
    p->mixed_precond = 1;
    p->t_tens = 0;
    p->cmu = 0.05;
    p->cdes = 0.65;
    p->lcar = 0.05715;
    p->sigma = 0.0728;
}

extern "C" int suli_field_shape(const suli_params *p, int f, int lo[3], int hi[3])
{
    if (!p || !lo || !hi) return fail(SULI_BAD_ARG, "null argument");
    const int nx = p->nx, ny = p->ny, nz = p->nz, nx1 = nx + 1, ny1 = ny + 1, nz1 = nz + 1;
    auto set = [&](int a, int b, int c, int d, int e, int g) {
        lo[0] = a; hi[0] = b; lo[1] = c; hi[1] = d; lo[2] = e; hi[2] = g;
    };
    switch (f) {
    case SULI_F_U: set(0, nx1 + 1, 0, ny + 1, 0, nz + 1); break;
    case SULI_F_V: set(0, nx + 1, 0, ny1 + 1, 0, nz + 1); break;
    case SULI_F_W: set(0, nx + 1, 0, ny + 1, 0, nz1 + 1); break;
    case SULI_F_PRD1: case SULI_F_PRD: case SULI_F_KA: case SULI_F_PRD0:
        set(0, nx + 1, 0, ny + 1, 0, nz + 1); break;
    case SULI_F_LS: case SULI_F_HS: case SULI_F_RHO: case SULI_F_LS_MU: case SULI_F_MU: case SULI_F_MUT:
    case SULI_F_DIV: case SULI_F_OBS_LSS: case SULI_F_ID_IBM:
    case SULI_F_HSX: case SULI_F_HSY: case SULI_F_HSZ: case SULI_F_KURV: case SULI_F_NUT:
        set(1, nx, 1, ny, 1, nz); break;
    case SULI_F_XMU: case SULI_F_FU: case SULI_F_U0: case SULI_F_FU0: case SULI_F_FU1: case SULI_F_TF_U:
    case SULI_F_OBS_LSX: case SULI_F_ID_IBMX: case SULI_F_PX:
        set(1, nx1, 1, ny, 1, nz); break;
    case SULI_F_YMU: case SULI_F_FV: case SULI_F_V0: case SULI_F_FV0: case SULI_F_FV1: case SULI_F_TF_V:
    case SULI_F_OBS_LSY: case SULI_F_ID_IBMY: case SULI_F_PY:
        set(1, nx, 1, ny1, 1, nz); break;
    case SULI_F_ZMU: case SULI_F_FW: case SULI_F_W0: case SULI_F_FW0: case SULI_F_FW1: case SULI_F_TF_W:
    case SULI_F_OBS_LSZ: case SULI_F_ID_IBMZ: case SULI_F_PZ:
        set(1, nx, 1, ny, 1, nz1); break;
    case SULI_F_BXX0: case SULI_F_BXX1: case SULI_F_BXZ0: set(0, ny + 1, 0, nz + 1, 0, 0); break;
    case SULI_F_BLX1: set(1, ny, 1, nz, 0, 0); break;
    case SULI_F_OBS_LS: set(1, nx1, 1, ny1, 1, nz1); break;
    default: return fail(SULI_BAD_ARG, "unknown field id " + std::to_string(f));
    }
    return SULI_OK;
}

static bool is_int_field(int f)
{
    return f == SULI_F_ID_IBMX || f == SULI_F_ID_IBMY || f == SULI_F_ID_IBMZ || f == SULI_F_ID_IBM;
}
static bool is_plane_field(int f)
{
    return f == SULI_F_BXX0 || f == SULI_F_BXX1 || f == SULI_F_BLX1 || f == SULI_F_BXZ0;
}

static int validate(const suli_params &p)
{
    auto bad = [](const std::string &m) { return fail(SULI_BAD_CONFIG, m); };
    if (p.nx < 4 || p.ny < 4 || p.nz < 4) return bad("nx, ny, nz must be >= 4");
    if (!(p.dx > 0 && p.dy > 0 && p.dz > 0 && p.dt > 0)) return bad("dx, dy, dz, dt must be > 0");
    if (p.der != 3) return bad("only der = 3 (2nd-order upwind) is supported");
    if (p.adv_type != 1) return bad("only adv_type = 1 (classical advection) is supported");
    if (p.t_press != 1 && p.t_press != 2)
        return bad("t_press must be 1 (projection) or 2 (IPA); the hydrostatic t_press = 0 is not supported");
    if (p.m_turb < 0 || p.m_turb > 3) return bad("m_turb must be 0..3");
    if (p.m_turb >= 2 && !(p.lcar > 0 && p.cmu >= 0 && p.cdes > 0)) return bad("m_turb >= 2 needs lcar > 0, cmu >= 0, cdes > 0");
    if (p.mms_t != 0 && p.mms_t != 1) return bad("mms_t must be 0 or 1");
    if (p.ibm_t != 0 && p.ibm_t != 2) return bad("ibm_t must be 0 or 2 (image-point IBM)");
    if (p.ibm_t == 2 && p.obst_t == 0) return bad("ibm_t = 2 needs an obstacle (obst_t != 0, obstacle fields uploaded)");
    if (p.t_tempo < 0 || p.t_tempo > 4) return bad("t_tempo must be 0..4");
    if (p.precision != SULI_PREC_FP64 && p.precision != SULI_PREC_MIXED) return bad("precision must be 0 or 1");
    if (!(p.ccx0 >= 0 && p.ccx0 <= 4)) return bad("ccx0 must be 0..4");
    if (!(p.ccxf == 0 || p.ccxf == 1 || p.ccxf == 2 || p.ccxf == 4)) return bad("ccxf must be 0, 1, 2 or 4");
    if (p.ccy0 < 0 || p.ccy0 > 2 || p.ccyf < 0 || p.ccyf > 2) return bad("ccy0/ccyf must be 0, 1 or 2");
    if (p.ccz0 < 1 || p.ccz0 > 2 || p.cczf < 1 || p.cczf > 2) return bad("ccz0/cczf must be 1 or 2");
    if ((p.ccx0 == 0) != (p.ccxf == 0)) return bad("periodic x must be set at both ends");
    if ((p.ccy0 == 0) != (p.ccyf == 0)) return bad("periodic y must be set at both ends");
    if (p.reinit_max_iter < 1) return bad("reinit_max_iter must be >= 1");
    if (p.cg_max_iter < 1) return bad("cg_max_iter must be >= 1");
    if (p.t_tens != 0 && p.t_tens != 1) return bad("t_tens must be 0 or 1");
    if (p.esp_type < 0 || p.esp_type > 2) return bad("esp_type must be 0, 1 or 2");
    if (!(p.wave_t == 0 || p.wave_t == 1 || p.wave_t == 2 || p.wave_t == 5)) return bad("wave_t must be 0, 1, 2 or 5");
    if (p.wave_t > 0 && !(p.n_w > 0 && p.h0_f > 0)) return bad("wave_t > 0 needs waves_coef's n_w > 0 and h0_f > 0");
    if (p.dz_t != 0 && p.dz_t != 1) return bad("dz_t must be 0 (uniform) or 1 (linear, SuLi-ICdz)");
    if (p.dz_t == 1) {
        if (!(p.dzmin > 0 && p.dzmax > 0)) return bad("dz_t = 1 needs dzmin > 0 and dzmax > 0");
        if (p.m_turb != 0 || p.ibm_t != 0 || p.t_tens != 0 || p.t_press != 1 || p.mms_t != 0 || p.esp_type != 0 ||
            p.wave_t != 0 || p.ccx0 == 3)
            return bad("dz_t = 1 (variable dz) is built for the plain two-fluid flow: m_turb = 0, no IBM, surface "
                       "tension, IPA, MMS, sponge, waves or inflow");
    }
    if (p.outflow_flux != 0 && p.outflow_flux != 1) return bad("outflow_flux must be 0 or 1");
    if (p.outflow_flux == 1 && !(p.ccxf == 4 && p.ccx0 == 3))
        return bad("outflow_flux = 1 balances a free outflow (ccxf = 4) against a prescribed inflow (ccx0 = 3)");
    if ((long long)p.nx * p.ny * p.nz > (1LL << 31) - 1) return bad("grid larger than 2^31 cells");
    return SULI_OK;
}

// ---------------------------------------------------------------------------
struct ImplBase {
    virtual ~ImplBase() {}
    virtual int copy_field(int icase, int f, void *host, bool up) = 0;
    virtual int copy_fields(int n, const int32_t *cases, const int32_t *fields, void *const *hosts, bool up) = 0;
    virtual int heaviside_init() = 0;
    virtual int level_set() = 0;
    virtual int contorno(int nlock) = 0;
    virtual int visco() = 0;
    virtual int convdiff(int fuse) = 0;
    virtual int complementos() = 0;
    virtual int tempo() = 0;
    virtual int graddin(int32_t *iters) = 0;
    virtual int posdin() = 0;
    virtual int conmassa(double *maxdiv) = 0;
    virtual int mms_error(double *err) = 0;
    virtual int set_stage(int tt) = 0;
    virtual int step(int n) = 0;
    virtual int read_scalars() = 0;
    virtual int write_case_scalar(int icase, int slot, double v) = 0;
    virtual int sync() = 0;
    virtual int time_kernel(int kernel, int reps, double *ms, double *bytes) = 0;
    virtual int write_fields(int icase, const char *path, int t_plot) = 0;
    virtual int ibm_setup() = 0;
    virtual int exp_press() = 0;
    virtual int contorno_les() = 0;
    virtual bool stored(int icase, int f) = 0;
    virtual int boundary_waves() = 0;
    virtual int autotune(suli_tuning *out) = 0;
    virtual int get_tuning(suli_tuning *out) = 0;
    unsigned long long inflow_calls = 0;
    int ncases = 0;
    std::vector<suli_params> P;
    double *hsc = nullptr;   // pinned host mirror of the per-case scalars
    int it = 0, tt = 1, ntt = 1;
    double t = 0.0, dt = 0.0, dt0 = 0.0, a_dt[3] = {0, 0, 0};
    int cg_iters[3] = {0, 0, 0}, cg_outer[3] = {0, 0, 0};
    double cg_res[3] = {0, 0, 0};
    int prev_cg[3] = {8, 8, 8};
    int replay_cg[3] = {-1, -1, -1}, replay_reinit = -1;
    int reinit_iters = 0, vol_loops = 0;
    int warn = 0;
    // mixed form: the unit-dt FP64 pressure operator on the device matches
    // the current density (cleared by every call that may change it)
    bool op_valid = false;
    // the density changed: the projection's operator follows it; the IPA's
    // (t_press = 2, the constant density rho_f1) does not
    void density_changed()
    {
        if (P[0].t_press != 2) op_valid = false;
    }
    // measurement
    bool prof = false;
    unsigned long long launch0 = 0;
    double cg_ms = 0.0, cg_cell_iters = 0.0;
    virtual void *stream() = 0;
};

struct suli_handle {
    ImplBase *impl;
};

// Field transfer of the mixed form: the caller's FP64 block (reference
// layout, dense, e0 x e1 x e2 column-major) <-> the padded FP32 device box
// (row pitch `pitch`, `height` rows per plane, block origin lo0/lo1/lo2),
// converted on the GPU through an FP64 device staging buffer.
template <typename T>
__global__ void k_unpack_field(const double *__restrict__ src, T *__restrict__ box, long long n, int e0, int e1,
                               int lo0, int lo1, int lo2, long long pitch, long long height)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % e0);
        const long long r = t / e0;
        const int j = (int)(r % e1);
        const int k = (int)(r / e1);
        box[(lo0 + i) + pitch * ((lo1 + j) + height * (long long)(lo2 + k))] = T(src[t]);
    }
}

// the same into the FP32 box and, when master is not null, its FP64 master
// from one read of the source (the source may be pinned host memory read
// over the chip-to-chip link)
template <typename T>
__global__ void k_unpack_field2(const double *__restrict__ src, T *__restrict__ box, double *__restrict__ master,
                                long long n, int e0, int e1, int lo0, int lo1, int lo2, long long pitch, long long height)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % e0);
        const long long r = t / e0;
        const int j = (int)(r % e1);
        const int k = (int)(r / e1);
        const long long q = (lo0 + i) + pitch * ((lo1 + j) + height * (long long)(lo2 + k));
        const double v = src[t];
        box[q] = T(v);
        if (master) master[q] = v;
    }
}

// one field transfer of a list (mixed form, page-locked host side): mode 0
// host FP64 -> FP32 box (and FP64 master), 1 FP64 master -> host, 2 FP32 box
// -> host
template <typename T> struct XferDesc {
    double *host;
    T *box;
    double *master;
    int n, e0, e1, lo0, lo1, lo2, mode;
    long long pitch, height;
};

// every transfer of a list in one launch: blockIdx.y the transfer,
// blockIdx.x strides its elements
template <typename T>
__global__ void __launch_bounds__(256) k_xfer_list(const XferDesc<T> *__restrict__ ds)
{
    const XferDesc<T> d = ds[blockIdx.y];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < d.n; t += gridDim.x * blockDim.x) {
        const int i = t % d.e0;
        const int r = t / d.e0;
        const int j = r % d.e1;
        const int k = r / d.e1;
        const long long q = (d.lo0 + i) + d.pitch * ((d.lo1 + j) + d.height * (long long)(d.lo2 + k));
        if (d.mode == 0) {
            const double v = d.host[t];
            d.box[q] = T(v);
            if (d.master) d.master[q] = v;
        } else if (d.mode == 1) {
            d.host[t] = d.master[q];
        } else {
            d.host[t] = (double)d.box[q];
        }
    }
}

template <typename T>
__global__ void k_pack_field(const T *__restrict__ box, double *__restrict__ dst, long long n, int e0, int e1,
                             int lo0, int lo1, int lo2, long long pitch, long long height)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % e0);
        const long long r = t / e0;
        const int j = (int)(r % e1);
        const int k = (int)(r / e1);
        dst[t] = (double)box[(lo0 + i) + pitch * ((lo1 + j) + height * (long long)(lo2 + k))];
    }
}

template <typename T>
struct Impl : ImplBase {
    Batch<T> b;
    std::vector<CaseDev<T>> hc;
    std::vector<void *> slabs;
    double *dsc = nullptr, *dpart = nullptr, *drk = nullptr;
    unsigned *dcnt = nullptr, *dactdone = nullptr;
    int *dact = nullptr;
    double *dstage = nullptr;      // mixed form: FP64 staging of field transfers
    void *dxfer = nullptr, *hxfer = nullptr;   // transfer-list descriptors (device, pinned host)
    size_t xfer_cap = 0;
    size_t stage_elems = 0;
    // One preconditioned CG iteration (about 75 kernels: product, update,
    // V-cycle, r.z, direction) captured per active-table slot and replayed:
    // the launches are the same every iteration (fixed device pointers and
    // grids), only the data they find differs.  Captured after an iteration
    // has run uncaptured (the one-time grid queries are done by then).
    cudaGraphExec_t pcg_graph[2] = {nullptr, nullptr};
    unsigned long long pcg_graph_kernels = 0;
    bool pcg_plain_done = false;
    int use_graphs = -1;

    // n preconditioned iterations from table `slot`; returns the current slot
    int pcg_iters(int n, int slot)
    {
        if (use_graphs < 0) {
            const char *env = std::getenv("SULI_GRAPHS");
            use_graphs = (env && std::string(env) == "0") ? 0 : 1;
        }
        if (!use_graphs || !pcg_plain_done) {
            slot = launch_pcg_iters<T>(b, n, slot, st);
            pcg_plain_done = true;
            return slot;
        }
        for (int q = 0; q < n; ++q) {
            if (!pcg_graph[slot]) {
                const unsigned long long before = g_launches.load();
                cudaGraph_t graph = nullptr;
                if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                    cudaGetLastError();
                    use_graphs = 0;
                    return launch_pcg_iters<T>(b, n - q, slot, st);
                }
                launch_pcg_iters<T>(b, 1, slot, st);
                cudaError_t e = cudaStreamEndCapture(st, &graph);
                const unsigned long long captured = g_launches.load() - before;
                g_launches.fetch_sub(captured);   // captured launches have not run
                if (e != cudaSuccess || cudaGraphInstantiate(&pcg_graph[slot], graph, 0) != cudaSuccess) {
                    cudaGetLastError();
                    if (graph) cudaGraphDestroy(graph);
                    pcg_graph[slot] = nullptr;
                    use_graphs = 0;
                    return launch_pcg_iters<T>(b, n - q, slot, st);
                }
                cudaGraphDestroy(graph);
                pcg_graph_kernels = captured;
            }
            if (cudaGraphLaunch(pcg_graph[slot], st) != cudaSuccess) return -1;
            count_launch(pcg_graph_kernels);
            slot = 1 - slot;
        }
        return slot;
    }
    // ---- the whole time step as one CUDA graph -------------------------------
    // Mixed form with multigrid passes (the ensemble's configuration): the
    // loops the host drove by reading scalars -- the volume correction, the
    // FP64 refinement passes of each graddin and the FP32 iterations inside
    // a pass -- are conditional WHILE nodes whose conditions k_loop_cond sets
    // from the same scalars (every loop also capped on the device); the
    // straight-line stretches between them are captured launches.  Built
    // once per handle, after the autotuner, and replayed every step: one
    // launch and one host read per step.  SULI_STEP_GRAPH=0 keeps the host-
    // driven step; configurations whose launches carry per-step host values
    // (replayed counts, the manufactured solution, the IPA, the waves) keep
    // it too; the step number and the inflow's random-number call count,
    // which the AB schemes and the inflow take, are copied into case 0's
    // scalars before each launch and read there (the waves' time likewise,
    // should they join).  Iterations past a case's convergence are no-ops (it has left the
    // active tables), so both paths give the same bits.
    cudaGraphExec_t step_exec = nullptr;
    int step_graph_state = 0;      // 0 not built, 1 built, -1 not used by this handle
    bool sg_capturing = false;     // launches read the step's host values from case 0's scalars
    unsigned long long sg_rng_per_step = 0;   // inflow calls of one step
    double *sg_hvals = nullptr;    // pinned: the step number, time and inflow call count of the step
    unsigned long long sg_static = 0, sg_vol = 0, sg_outer[3] = {0, 0, 0}, sg_inner[3] = {0, 0, 0};

    bool graphs_enabled()
    {
        if (use_graphs < 0) {
            const char *env = std::getenv("SULI_GRAPHS");
            use_graphs = (env && std::string(env) == "0") ? 0 : 1;
        }
        return use_graphs == 1;
    }
    bool step_graph_eligible()
    {
        const char *env = std::getenv("SULI_STEP_GRAPH");
        if (env && std::string(env) == "0") return false;
        if (sizeof(T) != 4 || b.nlev < 2 || !graphs_enabled() || use_cluster()) return false;
        if (P[0].t_press != 1) return false;
        if (replay_reinit >= 0) return false;
        for (int q = 0; q < 3; ++q)
            if (replay_cg[q] >= 0) return false;
        for (const auto &q : P)
            if (q.mms_t != 0 || q.wave_t > 0) return false;
        if (!tuned && tune_env == 1) return false;
        return step_graph_eligible_shape();
    }
    // the configuration conditions of the step graph (not whether the
    // autotuner has run)
    bool step_graph_eligible_shape()
    {
        const char *env = std::getenv("SULI_STEP_GRAPH");
        if (env && std::string(env) == "0") return false;
        if (sizeof(T) != 4 || b.nlev < 2 || !graphs_enabled() || use_cluster()) return false;
        if (P[0].t_press != 1) return false;
        if (replay_reinit >= 0) return false;
        for (int q = 0; q < 3; ++q)
            if (replay_cg[q] >= 0) return false;
        for (const auto &q : P)
            if (q.mms_t != 0 || q.wave_t > 0) return false;
        return true;
    }
    // the launches fn makes on st, captured into a graph (they have not run:
    // their count leaves the launch counter and comes back in n)
    template <class F> cudaGraph_t capture_seg(F fn, unsigned long long &n)
    {
        const unsigned long long before = g_launches.load();
        cudaGraph_t gph = nullptr;
        n = 0;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        const int rc = fn();
        const cudaError_t e = cudaStreamEndCapture(st, &gph);
        n = g_launches.load() - before;
        g_launches.fetch_sub(n);
        if (rc != SULI_OK || e != cudaSuccess) {
            cudaGetLastError();
            if (gph) cudaGraphDestroy(gph);
            return nullptr;
        }
        return gph;
    }
    // child graph `child` appended to g after node `last`
    static bool add_child(cudaGraph_t g, cudaGraphNode_t &last, cudaGraph_t child)
    {
        if (!child) return false;
        cudaGraphNode_t nd = nullptr;
        const bool ok = cudaGraphAddChildGraphNode(&nd, g, last ? &last : nullptr, last ? 1 : 0, child) == cudaSuccess;
        cudaGraphDestroy(child);
        if (ok) last = nd;
        return ok;
    }
    // a WHILE node on handle h appended to g after `last`; its body in *body
    static bool add_while(cudaGraph_t g, cudaGraphNode_t &last, cudaGraphConditionalHandle h, cudaGraph_t *body)
    {
        // (the parameter union has no default constructor: zeroed storage)
        alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
        std::memset(raw, 0, sizeof(raw));
        cudaGraphNodeParams *p = reinterpret_cast<cudaGraphNodeParams *>(raw);
        p->type = cudaGraphNodeTypeConditional;
        p->conditional.handle = h;
        p->conditional.type = cudaGraphCondTypeWhile;
        p->conditional.size = 1;
        cudaGraphNode_t nd = nullptr;
        if (cudaGraphAddNode(&nd, g, last ? &last : nullptr, nullptr, last ? 1 : 0, p) != cudaSuccess) return false;
        *body = p->conditional.phGraph_out[0];
        last = nd;
        return true;
    }
    // the step's launches up to the first solve's loops, or between loops,
    // as the host-driven step() makes them (no host reads)
    int sg_level_set(cudaGraphConditionalHandle hvol)
    {
        launch_step_reset<T>(b, st);
        density_changed();
        int rc;
        if ((rc = setsc(S_DTADV, dt))) return rc;
        if ((rc = setsc(S_RINREPLAY, -1.0))) return rc;
        launch_level_set_adv<T>(b, st);
        launch_reinit<T>(b, P[0].reinit_max_iter, st);
        launch_heaviside<T>(b, 0, st);
        launch_loop_cond<T>(b, 2, S_TRIP_VOL, (double)P[0].vol_loop_max, hvol, st);
        CKL();
        return SULI_OK;
    }
    // stage q up to its solve's passes
    int sg_stage_head(int q, cudaGraphConditionalHandle hout)
    {
        if constexpr (sizeof(T) != 4) return SULI_BAD_CONFIG;   // the mixed form's step only
        int rc;
        if ((rc = set_stage(q))) return rc;
        if ((rc = convdiff(1))) return rc;
        if ((rc = tempo())) return rc;
        if ((rc = boundary_waves())) return rc;
        if ((rc = contorno(2))) return rc;
        if ((rc = setsc(S_CGREPLAY, -1.0))) return rc;
        if (!op_valid) {
            launch_cg_refine_operator<T>(b, st);
            launch_mg_coarsen<T>(b, st);
            op_valid = true;
        }
        launch_cg_refine_setup<T>(b, st);
        launch_loop_cond<T>(b, 1, S_TRIP_OUT0 + q - 1, 64.0, hout, st);
        CKL();
        return SULI_OK;
    }
    int sg_build()
    {
        if constexpr (sizeof(T) != 4) return -1;   // the mixed form's step only
        const int cgmax = P[0].cg_max_iter;
        const double cap_pairs = (double)((cgmax + 256) / 2 + 1);
        cudaGraph_t G = nullptr;
        if (!sg_hvals && cudaMallocHost(&sg_hvals, 3 * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            sg_hvals = nullptr;
            return -1;
        }
        if (cudaGraphCreate(&G, 0) != cudaSuccess) return -1;
        // the captured launches take the step's host values from the device
        // (inflow calls counted from the start of the step)
        sg_capturing = true;
        const unsigned long long rng0 = inflow_calls;
        inflow_calls = 0;
        bool ok = true;
        cudaGraphNode_t last = nullptr;
        unsigned long long n = 0;
        sg_static = 0;
        cudaGraphConditionalHandle hvol;
        ok = ok && cudaGraphConditionalHandleCreate(&hvol, G, 0, cudaGraphCondAssignDefault) == cudaSuccess;
        ok = ok && add_child(G, last, capture_seg([&] { return sg_level_set(hvol); }, n));
        sg_static += n;
        cudaGraph_t vbody = nullptr;
        ok = ok && add_while(G, last, hvol, &vbody);
        if (ok) {
            cudaGraphNode_t vl = nullptr;
            ok = add_child(vbody, vl, capture_seg([&] {
                launch_volcorr<T>(b, st);
                launch_loop_cond<T>(b, 2, S_TRIP_VOL, (double)P[0].vol_loop_max, hvol, st);
                CKL();
                return SULI_OK;
            }, n));
            sg_vol = n;
        }
        for (int q = 1; q <= ntt && ok; ++q) {
            const int si = q - 1;
            cudaGraphConditionalHandle hout;
            ok = cudaGraphConditionalHandleCreate(&hout, G, 0, cudaGraphCondAssignDefault) == cudaSuccess;
            ok = ok && add_child(G, last, capture_seg([&] {
                int rc;
                if (q == 1) {
                    if (any_tens()) launch_curvature<T>(b, st);   // after the volume correction
                    if ((rc = contorno(3))) return rc;
                    if ((rc = visco())) return rc;
                }
                return sg_stage_head(q, hout);
            }, n));
            sg_static += n;
            cudaGraph_t obody = nullptr;
            ok = ok && add_while(G, last, hout, &obody);
            if (!ok) break;
            cudaGraphNode_t ol = nullptr;
            cudaGraphConditionalHandle hin;
            ok = cudaGraphConditionalHandleCreate(&hin, obody, 0, cudaGraphCondAssignDefault) == cudaSuccess;
            unsigned long long n1 = 0, n2 = 0;
            ok = ok && add_child(obody, ol, capture_seg([&] {
                launch_cg_table<T>(b, 0, st);
                launch_pcg_start<T>(b, 0, st);
                launch_loop_cond<T>(b, 0, S_TRIP_IN0 + si, cap_pairs, hin, st);
                CKL();
                return SULI_OK;
            }, n1));
            cudaGraph_t ibody = nullptr;
            ok = ok && add_while(obody, ol, hin, &ibody);
            if (!ok) break;
            cudaGraphNode_t il = nullptr;
            ok = add_child(ibody, il, capture_seg([&] {
                launch_pcg_iters<T>(b, 1, 0, st);
                launch_pcg_iters<T>(b, 1, 1, st);
                launch_loop_cond<T>(b, 0, S_TRIP_IN0 + si, cap_pairs, hin, st);
                CKL();
                return SULI_OK;
            }, n));
            sg_inner[si] = n;
            ok = ok && add_child(obody, ol, capture_seg([&] {
                launch_cg_refine_next<T>(b, st);
                launch_loop_cond<T>(b, 1, S_TRIP_OUT0 + si, 64.0, hout, st);
                CKL();
                return SULI_OK;
            }, n2));
            sg_outer[si] = n1 + n2;
            ok = ok && add_child(G, last, capture_seg([&] {
                launch_cg_refine_finish<T>(b, st);
                launch_stage_record<T>(b, si, st);
                int rc;
                if ((rc = posdin())) return rc;
                if ((rc = contorno(1))) return rc;
                if (q == ntt) launch_conmassa<T>(b, st);
                CKL();
                return SULI_OK;
            }, n));
            sg_static += n;
        }
        sg_capturing = false;
        sg_rng_per_step = inflow_calls;
        inflow_calls = rng0;
        if (ok) ok = cudaGraphInstantiate(&step_exec, G, 0) == cudaSuccess;
        cudaGraphDestroy(G);
        cudaGetLastError();
        if (!ok) {
            if (step_exec) { cudaGraphExecDestroy(step_exec); step_exec = nullptr; }
            return -1;
        }
        return 0;
    }
    // one time step by the step graph (built on first use)
    int step_by_graph()
    {
        if (!step_exec && sg_build() != 0) return -1;
        it = it + 1;
        t = t + dt;
        sg_hvals[0] = (double)it;
        sg_hvals[1] = t;
        sg_hvals[2] = (double)inflow_calls;
        CK(cudaMemcpyAsync(dsc + S_ITSTEP, sg_hvals, 3 * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaGraphLaunch(step_exec, st));
        inflow_calls += sg_rng_per_step;
        count_launch(sg_static);
        int rc;
        if ((rc = read_scalars())) return rc;
        unsigned long long dyn = (unsigned long long)sc(0, S_TRIP_VOL) * sg_vol;
        for (int si = 0; si < ntt; ++si)
            dyn += (unsigned long long)sc(0, S_TRIP_OUT0 + si) * sg_outer[si] +
                   (unsigned long long)sc(0, S_TRIP_IN0 + si) * sg_inner[si];
        count_launch(dyn);
        vol_loops = (int)sc(0, S_TRIP_VOL);
        reinit_iters = (int)sc(0, S_RINITER);
        for (int c = 0; c < ncases; ++c)
            if (sc(c, S_VOLACTIVE) != 0.0) warn |= (1 << SULI_VOL_LOOP_CAP);
        const int cgmax = P[0].cg_max_iter;
        for (int si = 0; si < ntt; ++si) {
            int maxit = 0, passes = 0;
            for (int c = 0; c < ncases; ++c) {
                maxit = std::max(maxit, (int)sc(c, S_STIT0 + si));
                passes = std::max(passes, (int)sc(c, S_STOUT0 + si));
                if (prof) cg_cell_iters += cells(c) * sc(c, S_STIT0 + si);
            }
            cg_iters[si] = maxit;
            cg_outer[si] = passes;
            prev_cg[si] = std::max(1, maxit / std::max(1, passes));
            if (maxit >= cgmax) warn |= (1 << SULI_CG_MAXITER);
        }
        cg_res[ntt - 1] = sc(0, S_RRTRUE) * dt;
        for (int c = 0; c < ncases; ++c)
            if (sc(c, S_STSTALL) != 0.0) warn |= (1 << SULI_CG_STALLED);
        return check_finite();
    }
    void drop_step_graph()
    {
        if (step_exec) { cudaGraphExecDestroy(step_exec); step_exec = nullptr; }
        step_graph_state = 0;
    }

    cudaStream_t st = nullptr;

    ~Impl() override
    {
        if (st) cudaStreamSynchronize(st);
        if (step_exec) cudaGraphExecDestroy(step_exec);
        if (sg_hvals) cudaFreeHost(sg_hvals);
        for (void *p : slabs) cudaFree(p);
        cudaFree(dsc);
        cudaFree(dpart);
        cudaFree(dcnt);
        cudaFree(dact);
        cudaFree(dactdone);
        cudaFree(dstage);
        cudaFree(dxfer);
        if (hxfer) cudaFreeHost(hxfer);
        for (auto &gx : pcg_graph)
            if (gx) cudaGraphExecDestroy(gx);
        cudaFree(drk);
        cudaFree(dtmaps);
        cudaFree(dtilecase);
        cudaFree(b.dcases);
        if (hsc) cudaFreeHost(hsc);
        cudaFree(out_dev);
        if (out_host) cudaFreeHost(out_host);
        if (st) cudaStreamDestroy(st);
    }

    // field output (PRTSCR record): device staging and pinned host buffers,
    // grown on demand
    float *out_dev = nullptr, *out_host = nullptr;
    size_t out_dev_cap = 0, out_host_cap = 0;

    int write_fields(int icase, const char *path, int t_plot) override
    {
        if (icase < 0 || icase >= ncases) return fail(SULI_BAD_ARG, "case index out of range");
        if (!path || (t_plot != 0 && t_plot != 1)) return fail(SULI_BAD_ARG, "bad path or t_plot (0 or 1)");
        const suli_params &q = P[icase];
        if (q.dz_t == 1) return fail(SULI_BAD_CONFIG, "the field record of a variable-dz grid (dz_t = 1) is not built");
        const long long nx1 = q.nx + 1, ny1 = q.ny + 1, nz1 = q.nz + 1;
        const long long n1 = nx1 * ny1 * nz1, nc = (long long)q.nx * q.ny * q.nz;
        const long long ndev = 4 * n1 + nc + (t_plot ? 6 * nc : 0), nf = 3 * n1 + ndev;
        if (nf * 4 > 2147483647LL) return fail(SULI_BAD_ARG, "the record exceeds one Fortran record (2^31 - 1 bytes)");
        if ((size_t)ndev > out_dev_cap) {
            cudaFree(out_dev);
            out_dev = nullptr;
            out_dev_cap = 0;
            CK(cudaMalloc(&out_dev, sizeof(float) * ndev));
            out_dev_cap = (size_t)ndev;
        }
        if ((size_t)nf > out_host_cap) {
            if (out_host) cudaFreeHost(out_host);
            out_host = nullptr;
            out_host_cap = 0;
            CK(cudaMallocHost(&out_host, sizeof(float) * nf));
            out_host_cap = (size_t)nf;
        }
        launch_prtscr<T>(b, icase, out_dev, t_plot, st);
        CK(cudaMemcpyAsync(out_host + 3 * n1, out_dev, sizeof(float) * ndev, cudaMemcpyDeviceToHost, st));
        // node coordinates while the copy is in flight: running sums from -dx,
        // -dy, -dz as the reference forms them (4_plot.f90:553-564)
        std::vector<double> x1(nx1 + 1), y1(ny1 + 1), z1(nz1 + 1);
        x1[0] = -q.dx; y1[0] = -q.dy; z1[0] = -q.dz;
        for (long long i = 1; i <= nx1; ++i) x1[i] = x1[i - 1] + q.dx;
        for (long long j = 1; j <= ny1; ++j) y1[j] = y1[j - 1] + q.dy;
        for (long long k = 1; k <= nz1; ++k) z1[k] = z1[k - 1] + q.dz;
        float *xo = out_host, *yo = out_host + n1, *zo = out_host + 2 * n1;
        for (long long k = 1, o = 0; k <= nz1; ++k)
            for (long long j = 1; j <= ny1; ++j)
                for (long long i = 1; i <= nx1; ++i, ++o) {
                    xo[o] = (float)x1[i];
                    yo[o] = (float)y1[j];
                    zo[o] = (float)z1[k];
                }
        CK(cudaStreamSynchronize(st));
        CKL();
        std::FILE *fp = std::fopen(path, "wb");
        if (!fp) return fail(SULI_BAD_ARG, std::string("cannot open ") + path);
        const int32_t len = (int32_t)(nf * 4);
        bool ok = std::fwrite(&len, 4, 1, fp) == 1 && std::fwrite(out_host, 4, (size_t)nf, fp) == (size_t)nf &&
                  std::fwrite(&len, 4, 1, fp) == 1;
        ok = (std::fclose(fp) == 0) && ok;
        if (!ok) return fail(SULI_BAD_ARG, std::string("writing ") + path + " failed");
        return SULI_OK;
    }

    int create(const suli_params *p, int n)
    {
        ncases = n;
        P.assign(p, p + n);
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        hc.resize(n);
        int tiles = 0, chunks = 0, maxplane = 1, cd_units_total[3] = {0, 0, 0};
        long long cd_shell_total = 0;
        for (int c = 0; c < n; ++c) {
            const suli_params &q = P[c];
            CaseDev<T> &cd = hc[c];
            std::memset(&cd, 0, sizeof(cd));
            Geo &g = cd.g;
            g.nx = q.nx; g.ny = q.ny; g.nz = q.nz;
            g.sx = (q.nx + 3 + 7) / 8 * 8;
            g.sxy = g.sx * (q.ny + 3);
            g.total = g.sxy * (q.nz + 3);
            if (g.total >= (1LL << 31)) return fail(SULI_BAD_CONFIG, "a case's grid exceeds 2^31 padded cells");
            cd.ntx = (q.nx + 1 + TX - 1) / TX;
            cd.nty = (q.ny + 1 + TY - 1) / TY;
            cd.ntz = (q.nz + 1 + TZ - 1) / TZ;
            cd.ntiles = cd.ntx * cd.nty * cd.ntz;
            cd.tile_begin = tiles;
            tiles += cd.ntiles;
            cd.nchunks = col_units(q.nx, q.ny, q.nz);
            cd.chunk_begin = chunks;
            chunks += cd.nchunks;
            for (int v = 0; v < 3; ++v) {
                cd.cd_begin[v] = cd_units_total[v];
                cd_units_total[v] += convdiff_units(q.nx, q.ny, q.nz, v);
            }
            cd.cd_shell_begin = cd_shell_total;
            cd_shell_total += convdiff_shell_positions(q.nx, q.ny, q.nz);
            long long mp = std::max({(long long)(q.nx + 3) * (q.nz + 3), (long long)(q.nx + 3) * (q.ny + 3),
                                     (long long)(q.ny + 3) * (q.nz + 3),
                                     (long long)(q.nx + 2) * (q.nz + 2) + (long long)(q.nx + 2) * (q.ny + 2) +
                                         (long long)(q.ny + 2) * (q.nz + 2)});
            maxplane = (int)std::max<long long>(maxplane, mp);
            cd.dx = q.dx; cd.dy = q.dy; cd.dz = (q.dz_t == 1) ? q.dzmin : q.dz;   // dza of SuLi-ICdz
            cd.dx1 = std::max({q.dx, q.dy, cd.dz});
            cd.dt1 = 0.1 * cd.dx1;
            cd.deltai = std::pow(q.dx * q.dy * cd.dz, 1. / 3.);
            cd.idx = 1.0 / q.dx; cd.idy = 1.0 / q.dy; cd.idz = 1.0 / cd.dz;
            cd.fidx = (float)cd.idx; cd.fidy = (float)cd.idy; cd.fidz = (float)cd.idz;
            cd.alpha1 = q.alpha1;
            cd.rho_f1 = q.rho_f1; cd.mu_f1 = q.mu_f1; cd.rho_f2 = q.rho_f2; cd.mu_f2 = q.mu_f2;
            cd.gx = q.gx; cd.gz = q.gz;
            cd.cles = std::pow(q.dx * q.dy * q.dz, 2. / 3.) * q.csmag * q.csmag;
            cd.pi = std::acos(-1.0);
            cd.uinicial = q.uinicial; cd.iturb = q.iturb; cd.seed = q.seed;
            cd.ccx0 = q.ccx0; cd.ccxf = q.ccxf; cd.ccy0 = q.ccy0; cd.ccyf = q.ccyf; cd.ccz0 = q.ccz0; cd.cczf = q.cczf;
            cd.t_tempo = q.t_tempo; cd.m_turb = q.m_turb; cd.mms_t = q.mms_t; cd.ibm_t = q.ibm_t; cd.obst_t = q.obst_t;
            cd.t_tens = q.t_tens; cd.sigma = q.sigma;
            cd.cmu = q.cmu; cd.cdes = q.cdes; cd.lcar = q.lcar; cd.delta = cd.dx1;
            cd.t_press = q.t_press;
            cd.esp_type = q.esp_type;
            cd.wave_t = q.wave_t;
            cd.outflow_flux = q.outflow_flux;
            cd.a_w = q.a_w; cd.f_w = q.f_w; cd.n_w = q.n_w; cd.h0_f = q.h0_f;
            for (int m = 0; m < 5; ++m) { cd.aeta[m] = q.aeta[m]; cd.avel[m] = q.avel[m]; }
            cd.ipa = (q.t_press == 2 && (q.mms_t == 0 || q.project_under_mms)) ? 1 : 0;
            cd.reinit_max = q.reinit_max_iter; cd.cg_max = q.cg_max_iter; cd.cg_tol_mode = q.cg_tol_mode;
            cd.cg_tol = q.cg_tol;
            // one slab per case: every field of the case in the common box layout
            const size_t fb = ((size_t)g.total * sizeof(T) + 255) / 256 * 256;
            const size_t ib = ((size_t)g.total * sizeof(int) + 255) / 256 * 256;
            const size_t db = ((size_t)g.total * sizeof(double) + 255) / 256 * 256;
            const size_t pb = ((size_t)(q.ny + 3) * (q.nz + 3) * sizeof(T) + 255) / 256 * 256;
            T **tf[] = {&cd.u, &cd.v, &cd.w, &cd.prd1, &cd.prd, &cd.ls, &cd.lsb, &cd.lsc, &cd.funcs, &cd.hs,
                        &cd.rho, &cd.ls_mu, &cd.mu, &cd.mut, &cd.xmu, &cd.ymu, &cd.zmu, &cd.Fu, &cd.Fv, &cd.Fw,
                        &cd.u0, &cd.v0, &cd.w0, &cd.fu0, &cd.fv0, &cd.fw0, &cd.fu1, &cd.fv1, &cd.fw1, &cd.div,
                        &cd.tf_u, &cd.tf_v, &cd.tf_w, &cd.obs_lsx, &cd.obs_lsy, &cd.obs_lsz, &cd.obs_lss,
                        &cd.spi, &cd.spj, &cd.spk, &cd.dpr, &cd.e, &cd.r, &cd.p, &cd.mp, &cd.qpr, &cd.obs_ls,
                        &cd.hsx, &cd.hsy, &cd.hsz, &cd.kurv, &cd.nlx, &cd.nly, &cd.nlz};
            const int ntf = sizeof(tf) / sizeof(tf[0]);
            int **itf[] = {&cd.id_ibmx, &cd.id_ibmy, &cd.id_ibmz, &cd.id_ibm};
            T **ptf[] = {&cd.bxx0, &cd.bxx1, &cd.blx1, &cd.bxz0};
            const bool mixed = (sizeof(T) == 4);
            const bool mg = mixed && q.mixed_precond == 1;
            // k equation (m_turb >= 2) and IPA (t_press = 2) arrays only where used
            T **kf[] = {&cd.ka, &cd.nut, &cd.sij, &cd.ka0, &cd.fk0, &cd.fk1, &cd.fka};
            T **af[] = {&cd.prd0, &cd.px, &cd.py, &cd.pz};
            const int nkf = (q.m_turb >= 2) ? 7 : 0, naf = (q.t_press == 2) ? 4 : 0, nsf = (q.esp_type > 0) ? 1 : 0;
            // SuLi-ICdz's z spacing arrays (dz_t = 1): dz, dzz, 1/dz, 1/dzz over
            // 0..nz+1 and dz11 over -2..nz+3
            const size_t zb = (q.dz_t == 1) ? ((size_t)5 * (q.nz + 6) * sizeof(double) + 255) / 256 * 256 : 0;
            size_t bytes = fb * (ntf + nkf + naf + nsf) + ib * 4 + pb * 4 + (mixed ? 20 * db : 0) + (mg ? 8 * fb : 0) + zb;
            void *slab = nullptr;
            CK(cudaMalloc(&slab, bytes));
            slabs.push_back(slab);
            CK(cudaMemsetAsync(slab, 0, bytes, st));
            char *cur = (char *)slab;
            for (int f = 0; f < ntf; ++f) { *tf[f] = (T *)cur; cur += fb; }
            for (int f = 0; f < 4; ++f) { *itf[f] = (int *)cur; cur += ib; }
            for (int f = 0; f < 4; ++f) { *ptf[f] = (T *)cur; cur += pb; }
            for (int f = 0; f < nkf; ++f) { *kf[f] = (T *)cur; cur += fb; }
            for (int f = 0; f < naf; ++f) { *af[f] = (T *)cur; cur += fb; }
            if (nsf) { cd.epis = (T *)cur; cur += fb; }
            if (zb) {
                // dz_dist (SuLi-ICdz/2_iniciais.f90:326-406) and wenoz's extrapolated
                // spacing (SuLi-ICdz/8_derivadas.f90:1076-1084), formed on the host
                const int nz = q.nz, w = nz + 6;
                std::vector<double> hz((size_t)5 * w, 0.0);
                double *dzh = hz.data(), *dzzh = dzh + w, *idzh = dzzh + w, *idzzh = idzh + w, *d11 = idzzh + w + 2;
                for (int k = 0; k <= nz + 1; ++k) dzh[k] = q.dzmin + (q.dzmax - q.dzmin) * k / nz;
                for (int k = 1; k <= nz + 1; ++k) dzzh[k] = (dzh[k] + dzh[k - 1]) * 0.5;
                dzzh[0] = dzzh[1];
                dzzh[nz + 1] = dzzh[nz];
                for (int k = 0; k <= nz + 1; ++k) { idzh[k] = 1.0 / dzh[k]; idzzh[k] = 1.0 / dzzh[k]; }
                const double c11 = 1. / 11.;
                for (int k = 0; k <= nz + 1; ++k) d11[k] = dzh[k];
                d11[0] = c11 * (18. * d11[1] - 9. * d11[2] + 2. * d11[3]);
                d11[-1] = c11 * (18. * d11[0] - 9. * d11[1] + 2. * d11[2]);
                d11[-2] = c11 * (18. * d11[-1] - 9. * d11[0] + 2. * d11[1]);
                d11[nz + 1] = c11 * (18. * d11[nz] - 9. * d11[nz - 1] + 2. * d11[nz - 2]);
                d11[nz + 2] = c11 * (18. * d11[nz + 1] - 9. * d11[nz] + 2. * d11[nz - 1]);
                d11[nz + 3] = c11 * (18. * d11[nz + 2] - 9. * d11[nz + 1] + 2. * d11[nz]);
                double *dd = (double *)cur;
                CK(cudaMemcpyAsync(dd, hz.data(), sizeof(double) * hz.size(), cudaMemcpyHostToDevice, st));
                CK(cudaStreamSynchronize(st));   // the host vector dies with this scope
                cd.dzk = dd; cd.dzzk = dd + w; cd.idzk = dd + 2 * w; cd.idzzk = dd + 3 * w; cd.dz11 = dd + 4 * w + 2;
                cur += zb;
            }
            if (mixed) {
                double **d64[] = {&cd.e64, &cd.r64, &cd.rho64, &cd.spi64, &cd.spj64, &cd.spk64, &cd.dpr64, &cd.qpr64,
                                  &cd.u64, &cd.v64, &cd.w64, &cd.u064, &cd.v064, &cd.w064,
                                  &cd.ls64, &cd.lsb64, &cd.lsc64, &cd.pfx64, &cd.pfy64, &cd.pfz64};
                for (int f = 0; f < 20; ++f) { *d64[f] = (double *)cur; cur += db; }
            }
            if (mg) {
                // multigrid level 0: the case grid, its box and its tiles
                MgLev<T> &L = cd.mg[0];
                L.g = g;
                L.ntx = cd.ntx; L.nty = cd.nty; L.ntz = cd.ntz; L.ntiles = cd.ntiles;
                L.ncols = cd.nchunks;
                T **lf[] = {&L.cx, &L.cy, &L.cz, &L.dg, &L.z, &L.f, &L.z2, &L.dgi};
                for (int f = 0; f < 8; ++f) { *lf[f] = (T *)cur; cur += fb; }
            }
        }
        // multigrid levels: halve every dimension until the largest is at most
        // 4 in every case; all cases get the batch's level count
        int nlev = 1;
        if (sizeof(T) == 4 && P[0].mixed_precond == 1) {
            for (int c = 0; c < n; ++c) {
                int m = std::max({P[c].nx, P[c].ny, P[c].nz}), l = 1;
                while (m > 4 && l < MG_MAXL) { m = (m + 1) / 2; ++l; }
                nlev = std::max(nlev, l);
            }
            nlev = std::max(nlev, 2);
            for (int c = 0; c < n; ++c) {
                CaseDev<T> &cd = hc[c];
                cd.nlev = nlev;
                size_t bytes = 0;
                int dx = cd.g.nx, dy = cd.g.ny, dz = cd.g.nz;
                for (int l = 1; l < nlev; ++l) {
                    dx = (dx + 1) / 2; dy = (dy + 1) / 2; dz = (dz + 1) / 2;
                    MgLev<T> &L = cd.mg[l];
                    L.g.nx = dx; L.g.ny = dy; L.g.nz = dz;
                    L.g.sx = (dx + 3 + 7) / 8 * 8;
                    L.g.sxy = L.g.sx * (dy + 3);
                    L.g.total = L.g.sxy * (dz + 3);
                    L.ntx = (dx + TX - 1) / TX; L.nty = (dy + TY - 1) / TY; L.ntz = (dz + TZ - 1) / TZ;
                    L.ntiles = L.ntx * L.nty * L.ntz;
                    L.ncols = col_units(dx, dy, dz);
                    bytes += 8 * (((size_t)L.g.total * sizeof(T) + 255) / 256 * 256);
                    b.mg_tiles[l] += L.ntiles;
                }
                void *slab = nullptr;
                CK(cudaMalloc(&slab, bytes));
                slabs.push_back(slab);
                CK(cudaMemsetAsync(slab, 0, bytes, st));
                char *cur = (char *)slab;
                for (int l = 1; l < nlev; ++l) {
                    MgLev<T> &L = cd.mg[l];
                    const size_t lb = ((size_t)L.g.total * sizeof(T) + 255) / 256 * 256;
                    T **lf[] = {&L.cx, &L.cy, &L.cz, &L.dg, &L.z, &L.f, &L.dgi, &L.z2};
                    for (int f = 0; f < 8; ++f) { *lf[f] = (T *)cur; cur += lb; }
                }
            }
        }
        b.nlev = nlev;
        b.ncases = n;
        b.total_tiles = tiles;
        b.total_units = chunks;
        b.max_plane = maxplane;
        for (int v = 0; v < 3; ++v) b.total_cd_units[v] = cd_units_total[v];
        b.total_cd_shell = cd_shell_total;
        CK(cudaMalloc(&dsc, sizeof(double) * S_NSCAL * n));
        CK(cudaMemsetAsync(dsc, 0, sizeof(double) * S_NSCAL * n, st));
        // reduction partials: one per tile (tile kernels) or one per warp of
        // a column unit (persistent kernels), whichever needs more
        const int pstride = std::max(tiles, chunks * (NTHREADS / 32));
        CK(cudaMalloc(&dpart, sizeof(double) * NSLOT * (size_t)pstride));
        CK(cudaMalloc(&dcnt, sizeof(unsigned) * n));
        CK(cudaMemsetAsync(dcnt, 0, sizeof(unsigned) * n, st));
        // tables 0 and 1: the CG iteration; table 2: single-kernel profiling
        CK(cudaMalloc(&dact, sizeof(int) * 3 * act_stride(n, nlev)));
        CK(cudaMemsetAsync(dact, 0, sizeof(int) * 3 * act_stride(n, nlev), st));
        CK(cudaMalloc(&dactdone, sizeof(unsigned)));
        CK(cudaMemsetAsync(dactdone, 0, sizeof(unsigned), st));
        b.act = dact;
        b.act_done = dactdone;
        if (sizeof(T) != sizeof(double)) {
            for (int c = 0; c < n; ++c)
                stage_elems = std::max(stage_elems, (size_t)(P[c].nx + 3) * (P[c].ny + 3) * (P[c].nz + 3));
            CK(cudaMalloc(&dstage, stage_elems * sizeof(double)));
        }
        CK(cudaMallocHost(&hsc, sizeof(double) * S_NSCAL * n));
        double rk[9] = {1., 3. / 4., 1. / 3., 0., 1. / 4., 2. / 3., 1., 1. / 4., 2. / 3.};
        CK(cudaMalloc(&drk, sizeof(rk)));
        CK(cudaMemcpyAsync(drk, rk, sizeof(rk), cudaMemcpyHostToDevice, st));
        b.drk = drk;
        for (int c = 0; c < n; ++c) {
            hc[c].sc = dsc + (size_t)c * S_NSCAL;
            hc[c].partials = dpart;
            hc[c].pstride = pstride;
            hc[c].counter = dcnt + c;
            hc[c].total_tiles = tiles;
        }
        // the case of every tile of the launch grid (one load instead of a
        // search per block)
        {
            std::vector<int> tc((size_t)tiles);
            for (int c = 0; c < n; ++c)
                for (int t = 0; t < hc[c].ntiles; ++t) tc[(size_t)hc[c].tile_begin + t] = c;
            CK(cudaMalloc(&dtilecase, sizeof(int) * (size_t)std::max(tiles, 1)));
            CK(cudaMemcpyAsync(dtilecase, tc.data(), sizeof(int) * tc.size(), cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));
            for (int c = 0; c < n; ++c) hc[c].tile_case = dtilecase;
        }
        CK(cudaMalloc(&b.dcases, sizeof(CaseDev<T>) * n));
        CK(cudaMemcpyAsync(b.dcases, hc.data(), sizeof(CaseDev<T>) * n, cudaMemcpyHostToDevice, st));
        b.hcases = hc.data();
        if (int rc = make_tensor_maps()) return rc;
        tune_defaults();
        // time-integration coefficients, coef_tempo (2_iniciais.f90:278-312)
        dt0 = dt = P[0].dt;
        if (P[0].t_tempo == 1 || P[0].t_tempo == 2) {
            ntt = (P[0].t_tempo == 1) ? 2 : 3;
            a_dt[0] = 0.5 * dt; a_dt[1] = 1.0 * dt; a_dt[2] = 1.0 * dt;
        } else {
            ntt = 1;
            a_dt[0] = a_dt[1] = a_dt[2] = 1.0 * dt;
        }
        for (int c = 0; c < n; ++c) setsc_host_init(c);
        CK(cudaMemcpyAsync(dsc, hsc, sizeof(double) * S_NSCAL * n, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        return SULI_OK;
    }

    // Tensor maps of the TMA-staged convdiff: per case u, v, w, rho, mu, xmu,
    // ymu, zmu, each its padded box (sx x (ny+3) x (nz+3) elements, x
    // unit-stride) read in boxes of 40 x 12 x 1; out-of-box elements load as
    // zeros.  Without the CUDA driver's encoder (or with SULI_CONVDIFF=0) the
    // gather kernel runs instead.
    CUtensorMap *dtmaps = nullptr;
    int *dtilecase = nullptr;
    // the CUDA driver's tensor-map encoder (null when the CUDA driver has none)
    static PFN_cuTensorMapEncodeTiled_v12000 tensor_encoder()
    {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult qr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr) !=
                cudaSuccess || qr != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return nullptr;
        }
        return (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    int make_tensor_maps()
    {
        const char *env = std::getenv("SULI_CONVDIFF");
        if (env && std::string(env) == "0") return SULI_OK;
        for (int c = 0; c < ncases; ++c)
            if (P[c].dz_t == 1) return SULI_OK;   // the variable-dz stencils run in the gather kernel
        auto encode = tensor_encoder();
        if (!encode) return SULI_OK;
        std::vector<CUtensorMap> maps((size_t)ncases * 8);
        for (int c = 0; c < ncases; ++c) {
            const CaseDev<T> &cd = hc[c];
            const T *arr[8] = {cd.u, cd.v, cd.w, cd.rho, cd.mu, cd.xmu, cd.ymu, cd.zmu};
            const cuuint64_t dims[3] = {(cuuint64_t)cd.g.sx, (cuuint64_t)(cd.g.ny + 3), (cuuint64_t)(cd.g.nz + 3)};
            const cuuint64_t strides[2] = {(cuuint64_t)cd.g.sx * sizeof(T), (cuuint64_t)cd.g.sxy * sizeof(T)};
            const cuuint32_t box[3] = {(cuuint32_t)CD_MAP_BOX_X, (cuuint32_t)CD_MAP_BOX_Y, 1};
            const cuuint32_t estr[3] = {1, 1, 1};
            for (int a = 0; a < 8; ++a) {
                CUresult r = encode(&maps[(size_t)c * 8 + a],
                                    sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                                    (void *)arr[a], dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
                if (r != CUDA_SUCCESS) return SULI_OK;   // no maps: the gather kernel runs
            }
        }
        CK(cudaMalloc(&dtmaps, sizeof(CUtensorMap) * maps.size()));
        CK(cudaMemcpyAsync(dtmaps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        b.tmaps = dtmaps;
        // failure-path test hook: the staged convdiff's bounded TMA waits run
        // out once per case (reported as SULI_DEVICE_TIMEOUT)
        const char *e = std::getenv("SULI_TEST_TMA_SHORTFALL");
        b.test_shortfall = (e && std::atoi(e) == 1) ? 1 : 0;
        return SULI_OK;
    }

    void setsc_host_init(int c)
    {
        double *s = hsc + (size_t)c * S_NSCAL;
        std::memset(s, 0, sizeof(double) * S_NSCAL);
        s[S_DT] = dt;
        s[S_IDT] = (dt != 0.0) ? 1.0 / dt : 0.0;
        s[S_DTADV] = dt;
        s[S_RINREPLAY] = -1.0;
        s[S_CGREPLAY] = -1.0;
        s[S_CGMAX] = (double)P[c].cg_max_iter;
    }

    int setsc(int slot, double v)
    {
        launch_set_scalar<T>(b, slot, v, st);
        CKL();
        return SULI_OK;
    }

    int read_scalars() override
    {
        CK(cudaMemcpyAsync(hsc, dsc, sizeof(double) * S_NSCAL * ncases, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        return SULI_OK;
    }
    double sc(int c, int slot) const { return hsc[(size_t)c * S_NSCAL + slot]; }

    int write_case_scalar(int icase, int slot, double v) override
    {
        CK(cudaStreamSynchronize(st));
        CK(cudaMemcpy(dsc + (size_t)icase * S_NSCAL + slot, &v, sizeof(double), cudaMemcpyHostToDevice));
        hsc[(size_t)icase * S_NSCAL + slot] = v;
        return SULI_OK;
    }

    int sync() override
    {
        CK(cudaStreamSynchronize(st));
        return SULI_OK;
    }

    // one kernel alone over every case, `reps` launches between two events on
    // the library's stream (after two untimed launches)
    int time_kernel(int kernel, int reps, double *ms, double *bytes) override
    {
        if (reps < 1) return fail(SULI_BAD_ARG, "reps must be >= 1");
        if ((kernel == 1 || kernel == 3) && b.nlev < 2) return fail(SULI_BAD_ARG, "kernels 1 and 3 need the multigrid mixed form");
        if (launch_profile_kernel<T>(b, kernel, 1, st) != 0) return fail(SULI_BAD_ARG, "unknown kernel id");
        launch_profile_kernel<T>(b, kernel, 0, st);
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) launch_profile_kernel<T>(b, kernel, 0, st);
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        CKL();
        double cells = 0.0;
        for (int c = 0; c < ncases; ++c) cells += (double)P[c].nx * P[c].ny * P[c].nz;
        // algorithmic bytes per cell: A reads p and the three scaled
        // coefficients and writes mp (5 arrays); a red half-sweep streams z, f,
        // dg and the three conductances (shared cache lines: both colours) and
        // writes half of z (6.5); C reads r and p and writes p (3); a whole
        // one-pass sweep reads z, f, dg and the three conductances and writes
        // the other z buffer (7)
        const double per[4] = {5.0, 6.5, 3.0, 7.0};
        *ms = (double)t / reps;
        *bytes = cells * per[kernel] * (double)sizeof(T);
        return SULI_OK;
    }
    void *stream() override { return (void *)st; }
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int ev_begin()
    {
        if (!prof) return SULI_OK;
        if (!ev0) {
            CK(cudaEventCreate(&ev0));
            CK(cudaEventCreate(&ev1));
        }
        CK(cudaEventRecord(ev0, st));
        return SULI_OK;
    }
    int ev_end()
    {
        if (!prof) return SULI_OK;
        CK(cudaEventRecord(ev1, st));
        CK(cudaEventSynchronize(ev1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ev0, ev1));
        cg_ms += ms;
        return SULI_OK;
    }
    double cells(int c) const { return (double)P[c].nx * P[c].ny * P[c].nz; }

    // ---- field copies -------------------------------------------------------
    // FP64 master of a field (mixed form velocities), else null
    double *master_ptr(int icase, int f)
    {
        CaseDev<T> &c = hc[icase];
        switch (f) {
        case SULI_F_U: return c.u64;
        case SULI_F_V: return c.v64;
        case SULI_F_W: return c.w64;
        case SULI_F_U0: return c.u064;
        case SULI_F_V0: return c.v064;
        case SULI_F_W0: return c.w064;
        case SULI_F_LS: return c.ls64;
        default: return nullptr;
        }
    }

    void *dev_ptr(int icase, int f)
    {
        CaseDev<T> &c = hc[icase];
        switch (f) {
        case SULI_F_U: return c.u;
        case SULI_F_V: return c.v;
        case SULI_F_W: return c.w;
        case SULI_F_PRD1: return c.prd1;
        case SULI_F_PRD: return c.prd;
        case SULI_F_LS: return c.ls;
        case SULI_F_HS: return c.hs;
        case SULI_F_RHO: return c.rho;
        case SULI_F_LS_MU: return c.ls_mu;
        case SULI_F_MU: return c.mu;
        case SULI_F_MUT: return c.mut;
        case SULI_F_XMU: return c.xmu;
        case SULI_F_YMU: return c.ymu;
        case SULI_F_ZMU: return c.zmu;
        case SULI_F_FU: return c.Fu;
        case SULI_F_FV: return c.Fv;
        case SULI_F_FW: return c.Fw;
        case SULI_F_U0: return c.u0;
        case SULI_F_V0: return c.v0;
        case SULI_F_W0: return c.w0;
        case SULI_F_FU0: return c.fu0;
        case SULI_F_FV0: return c.fv0;
        case SULI_F_FW0: return c.fw0;
        case SULI_F_FU1: return c.fu1;
        case SULI_F_FV1: return c.fv1;
        case SULI_F_FW1: return c.fw1;
        case SULI_F_DIV: return c.div;
        case SULI_F_TF_U: return c.tf_u;
        case SULI_F_TF_V: return c.tf_v;
        case SULI_F_TF_W: return c.tf_w;
        case SULI_F_OBS_LSX: return c.obs_lsx;
        case SULI_F_OBS_LSY: return c.obs_lsy;
        case SULI_F_OBS_LSZ: return c.obs_lsz;
        case SULI_F_OBS_LSS: return c.obs_lss;
        case SULI_F_OBS_LS: return c.obs_ls;
        case SULI_F_HSX: return c.hsx;
        case SULI_F_HSY: return c.hsy;
        case SULI_F_HSZ: return c.hsz;
        case SULI_F_KURV: return c.kurv;
        case SULI_F_KA: return c.ka;
        case SULI_F_NUT: return c.nut;
        case SULI_F_PRD0: return c.prd0;
        case SULI_F_PX: return c.px;
        case SULI_F_PY: return c.py;
        case SULI_F_PZ: return c.pz;
        case SULI_F_ID_IBMX: return c.id_ibmx;
        case SULI_F_ID_IBMY: return c.id_ibmy;
        case SULI_F_ID_IBMZ: return c.id_ibmz;
        case SULI_F_ID_IBM: return c.id_ibm;
        case SULI_F_BXX0: return c.bxx0;
        case SULI_F_BXX1: return c.bxx1;
        case SULI_F_BXZ0: return c.bxz0;
        case SULI_F_BLX1: return c.blx1;
        default: return nullptr;
        }
    }

    // one field transfer, synchronous: the caller may reuse its buffer (or
    // read the data) once the call returns
    int copy_field(int icase, int f, void *host, bool up) override
    {
        if (up) op_valid = false;
        bool p64reset = false;
        int rc = enqueue_copy(icase, f, host, up, p64reset);
        if (rc) return rc;
        CK(cudaStreamSynchronize(st));
        // a pressure from the host replaces the FP64 pressure of the last solve
        if (p64reset) return write_case_scalar(icase, S_P64OK, 0.0);
        return SULI_OK;
    }

    // several transfers queued on the library's stream, one synchronisation
    int copy_fields(int n, const int32_t *cases, const int32_t *fields, void *const *hosts, bool up) override
    {
        if (n < 0 || (n > 0 && (!cases || !fields || !hosts))) return fail(SULI_BAD_ARG, "bad transfer list");
        if (up) op_valid = false;
        std::vector<int> reset;
        // mixed form: the transfers of FP32 fields whose host side is page-
        // locked go in one launch (k_xfer_list), the rest one by one
        std::vector<char> done(n, 0);
        if (sizeof(T) == 4 && n > 0) {
            std::vector<XferDesc<T>> ds;
            for (int q = 0; q < n; ++q) {
                if (!hosts[q] || cases[q] < 0 || cases[q] >= ncases || is_int_field(fields[q])) continue;
                double *hv = device_view(hosts[q]);
                void *dev = dev_ptr(cases[q], fields[q]);
                int lo[3], hi[3];
                if (!hv || !dev || suli_field_shape(&P[cases[q]], fields[q], lo, hi) != SULI_OK) continue;
                const Geo &g = hc[cases[q]].g;
                const long long e0 = hi[0] - lo[0] + 1, e1 = hi[1] - lo[1] + 1, e2 = hi[2] - lo[2] + 1;
                if (e0 * e1 * e2 >= (1LL << 31)) continue;
                XferDesc<T> d;
                d.host = hv;
                d.box = (T *)dev;
                d.master = master_ptr(cases[q], fields[q]);
                d.n = (int)(e0 * e1 * e2);
                d.e0 = (int)e0; d.e1 = (int)e1;
                d.lo0 = lo[0]; d.lo1 = lo[1]; d.lo2 = lo[2];
                d.mode = up ? 0 : (d.master ? 1 : 2);
                d.pitch = is_plane_field(fields[q]) ? (long long)(g.ny + 3) : (long long)g.sx;
                d.height = is_plane_field(fields[q]) ? (long long)(g.nz + 3) : (long long)(g.ny + 3);
                ds.push_back(d);
                done[q] = 1;
                if (up && fields[q] == SULI_F_PRD1) reset.push_back(cases[q]);
            }
            if (!ds.empty()) {
                const size_t bytes = sizeof(XferDesc<T>) * ds.size();
                if (bytes > xfer_cap) {
                    cudaFree(dxfer);
                    cudaFreeHost(hxfer);
                    dxfer = nullptr; hxfer = nullptr; xfer_cap = 0;
                    CK(cudaMalloc(&dxfer, bytes));
                    CK(cudaMallocHost(&hxfer, bytes));
                    xfer_cap = bytes;
                }
                std::memcpy(hxfer, ds.data(), bytes);
                CK(cudaMemcpyAsync(dxfer, hxfer, bytes, cudaMemcpyHostToDevice, st));
                for (size_t q0 = 0; q0 < ds.size(); q0 += 65535) {
                    const unsigned ny = (unsigned)std::min<size_t>(65535, ds.size() - q0);
                    k_xfer_list<T><<<dim3(64, ny), 256, 0, st>>>((const XferDesc<T> *)dxfer + q0);
                }
                CKL();
            }
        }
        for (int q = 0; q < n; ++q) {
            if (done[q]) continue;
            if (!hosts[q]) return fail(SULI_BAD_ARG, "null host pointer");
            bool p64reset = false;
            int rc = enqueue_copy(cases[q], fields[q], hosts[q], up, p64reset);
            if (rc) {
                cudaStreamSynchronize(st);
                return rc;
            }
            if (p64reset) reset.push_back(cases[q]);
        }
        CK(cudaStreamSynchronize(st));
        for (int c : reset) {
            int rc = write_case_scalar(c, S_P64OK, 0.0);
            if (rc) return rc;
        }
        return SULI_OK;
    }

    // the device's address of page-locked host memory (allocated or
    // registered through CUDA), or null for any other pointer (pageable
    // memory goes through the staging buffer)
    static double *device_view(void *host)
    {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
        return static_cast<double *>(a.devicePointer);
    }

    // queue one transfer on the library's stream (no synchronisation)
    int enqueue_copy(int icase, int f, void *host, bool up, bool &p64reset)
    {
        if (icase < 0 || icase >= ncases) return fail(SULI_BAD_ARG, "case index out of range");
        int lo[3], hi[3];
        int rc = suli_field_shape(&P[icase], f, lo, hi);
        if (rc) return rc;
        void *dev = dev_ptr(icase, f);
        if (!dev) return fail(SULI_BAD_ARG, "field not stored");
        const Geo &g = hc[icase].g;
        size_t e0 = hi[0] - lo[0] + 1, e1 = hi[1] - lo[1] + 1, e2 = hi[2] - lo[2] + 1;
        size_t n = e0 * e1 * e2;
        const bool isint = is_int_field(f);
        const size_t es = isint ? sizeof(int) : sizeof(T);
        size_t dpitch_el = is_plane_field(f) ? (size_t)(g.ny + 3) : (size_t)g.sx;
        size_t dheight = is_plane_field(f) ? (size_t)(g.nz + 3) : (size_t)(g.ny + 3);
        if (!isint && sizeof(T) != sizeof(double)) {
            // FP64 host block <-> FP32 box, converted on the GPU; velocities
            // also go to / come from their FP64 masters
            const int nb = (int)std::min<size_t>((n + 255) / 256, 4096);
            double *master = master_ptr(icase, f);
            // page-locked host memory the device can address: the conversion
            // kernel reads or writes it directly (no staging copy, so the
            // transfers of a list overlap on the link instead of queueing
            // behind one staging buffer)
            if (double *hv = device_view(host)) {
                if (up) {
                    k_unpack_field2<T><<<nb, 256, 0, st>>>(hv, (T *)dev, master, (long long)n, (int)e0, (int)e1, lo[0],
                                                           lo[1], lo[2], (long long)dpitch_el, (long long)dheight);
                    p64reset = (f == SULI_F_PRD1);
                } else if (master) {
                    k_pack_field<double><<<nb, 256, 0, st>>>(master, hv, (long long)n, (int)e0, (int)e1, lo[0], lo[1],
                                                             lo[2], (long long)dpitch_el, (long long)dheight);
                } else {
                    k_pack_field<T><<<nb, 256, 0, st>>>((const T *)dev, hv, (long long)n, (int)e0, (int)e1, lo[0], lo[1],
                                                        lo[2], (long long)dpitch_el, (long long)dheight);
                }
                CKL();
                return SULI_OK;
            }
            if (n > stage_elems) return fail(SULI_BAD_ARG, "field larger than the transfer staging buffer");
            if (up) {
                CK(cudaMemcpyAsync(dstage, host, n * sizeof(double), cudaMemcpyHostToDevice, st));
                k_unpack_field<T><<<nb, 256, 0, st>>>(dstage, (T *)dev, (long long)n, (int)e0, (int)e1, lo[0], lo[1],
                                                      lo[2], (long long)dpitch_el, (long long)dheight);
                if (master)
                    k_unpack_field<double><<<nb, 256, 0, st>>>(dstage, master, (long long)n, (int)e0, (int)e1, lo[0],
                                                               lo[1], lo[2], (long long)dpitch_el, (long long)dheight);
                CKL();
                p64reset = (f == SULI_F_PRD1);
            } else {
                if (master)
                    k_pack_field<double><<<nb, 256, 0, st>>>(master, dstage, (long long)n, (int)e0, (int)e1, lo[0],
                                                             lo[1], lo[2], (long long)dpitch_el, (long long)dheight);
                else
                    k_pack_field<T><<<nb, 256, 0, st>>>((const T *)dev, dstage, (long long)n, (int)e0, (int)e1, lo[0],
                                                        lo[1], lo[2], (long long)dpitch_el, (long long)dheight);
                CKL();
                CK(cudaMemcpyAsync(host, dstage, n * sizeof(double), cudaMemcpyDeviceToHost, st));
            }
            return SULI_OK;
        }
        void *hp = host;
        cudaMemcpy3DParms m;
        std::memset(&m, 0, sizeof(m));
        cudaPitchedPtr hpp = make_cudaPitchedPtr(hp, e0 * es, e0, e1);
        cudaPitchedPtr dpp = make_cudaPitchedPtr(dev, dpitch_el * es, dpitch_el, dheight);
        cudaPos pos = make_cudaPos((size_t)lo[0] * es, (size_t)lo[1], (size_t)lo[2]);
        m.extent = make_cudaExtent(e0 * es, e1, e2);
        if (up) {
            m.srcPtr = hpp;
            m.dstPtr = dpp;
            m.dstPos = pos;
            m.kind = cudaMemcpyHostToDevice;
        } else {
            m.srcPtr = dpp;
            m.srcPos = pos;
            m.dstPtr = hpp;
            m.kind = cudaMemcpyDeviceToHost;
        }
        CK(cudaMemcpy3DAsync(&m, st));
        return SULI_OK;
    }

    // ---- autotuner -------------------------------------------------------------
    bool tuned = false, tune_locked_mg = false;
    int tune_env = -1;                 // SULI_TUNE: 0 off
    double tune_default_ms = 0.0, tune_tuned_ms = 0.0;
    using TuneKey = std::tuple<int, int, int, long long, int>;   // device, precision, cases, cells, levels
    struct TuneVal { Tuning t; double dms, tms; };
    static std::map<TuneKey, TuneVal> &tune_cache()
    {
        static std::map<TuneKey, TuneVal> m;
        return m;
    }
    static std::mutex &tune_mu()
    {
        static std::mutex m;
        return m;
    }
    void tune_defaults()
    {
        // environment overrides, for comparisons and tests (SULI_MG_CTA_CELLS
        // also keeps the tuner off that knob; forced shapes switch it off)
        if (const char *e = std::getenv("SULI_MG_CTA_CELLS")) {
            b.tune.mg_block_cells = std::atoi(e);
            tune_locked_mg = true;
        }
        if (const char *e = std::getenv("SULI_TUNE_CD")) b.tune.cd_variant = std::max(0, std::min(2, std::atoi(e)));
        if (const char *e = std::getenv("SULI_TUNE_SWEEP")) b.tune.sweep_blocks_per_sm = std::max(0, std::atoi(e));
        const char *e = std::getenv("SULI_TUNE");
        tune_env = (e && std::atoi(e) == 0) ? 0 : 1;
        if (std::getenv("SULI_TUNE_CD") || std::getenv("SULI_TUNE_SWEEP")) tune_env = 0;
    }
    // mean time of `reps` calls of f on the stream, after one untimed call
    template <typename F> double time_it(F f, int reps)
    {
        f();
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps; ++r) f();
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return (double)ms / reps;
    }
    // as time_it, with the launches of f captured once into a graph and the
    // graph replayed (how the step graph runs them); falls back to time_it
    template <typename F> double time_graph(F f, int reps)
    {
        const unsigned long long before = g_launches.load();
        cudaGraph_t gph = nullptr;
        cudaGraphExec_t ex = nullptr;
        bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            f();
            ok = cudaStreamEndCapture(st, &gph) == cudaSuccess && gph &&
                 cudaGraphInstantiate(&ex, gph, 0) == cudaSuccess;
        }
        g_launches.store(before);   // captured, not run
        if (gph) cudaGraphDestroy(gph);
        if (!ok) {
            cudaGetLastError();
            if (ex) cudaGraphExecDestroy(ex);
            return time_it(f, reps);
        }
        const double ms = time_it([&] { cudaGraphLaunch(ex, st); }, reps);
        cudaGraphExecDestroy(ex);
        return ms;
    }
    void drop_graphs()
    {
        for (auto &gx : pcg_graph)
            if (gx) { cudaGraphExecDestroy(gx); gx = nullptr; }
        pcg_plain_done = false;
        drop_step_graph();
    }
    int autotune(suli_tuning *out) override
    {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        long long cells_all = 0;
        for (int c = 0; c < ncases; ++c) cells_all += (long long)P[c].nx * P[c].ny * P[c].nz;
        const TuneKey key{dev, (int)sizeof(T), ncases, cells_all, b.nlev};
        {
            std::lock_guard<std::mutex> lk(tune_mu());
            auto it = tune_cache().find(key);
            if (it != tune_cache().end()) {
                const int mgc = b.tune.mg_block_cells;
                b.tune = it->second.t;
                if (tune_locked_mg) b.tune.mg_block_cells = mgc;
                tune_default_ms = it->second.dms;
                tune_tuned_ms = it->second.tms;
                tuned = true;
                drop_graphs();
                return get_tuning(out);
            }
        }
        CK(cudaStreamSynchronize(st));
        const Tuning def;
        double dms = 0.0, tms = 0.0;
        // convdiff (+ complementos): planes per unit; writes only Fu, Fv, Fw,
        // which every stage recomputes before it reads them
        if (b.tmaps) {
            double best = 1e30;
            int bv = def.cd_variant;
            for (int v = 0; v < 3; ++v) {
                b.tune.cd_variant = v;
                const double ms = time_it([&] { launch_convdiff_tma<T>(b, 1, st); }, 3);
                if (v == def.cd_variant) dms += ms;
                if (ms < best) { best = ms; bv = v; }
            }
            b.tune.cd_variant = bv;
            tms += best;
        }
        // the multigrid V-cycle (mixed form): the coarse-end threshold, then
        // the level-0 sweep's blocks per SM; both on the all-case table and
        // touching only the V-cycle's own levels (rebuilt by the next solve)
        if (b.nlev > 1 && op_valid) {
            if (launch_profile_kernel<T>(b, 4, 1, st) != 0) return fail(SULI_CUDA_ERROR, "V-cycle timing");
            if (!tune_locked_mg) {
                double best = 1e30;
                int bc = def.mg_block_cells;
                // (inside a graph when the step runs as one: launches cost
                // little there, which moves the balance towards grid launches)
                const bool in_graph = step_graph_eligible_shape();
                for (int cells : {0, 4096, 16384, 65536}) {
                    b.tune.mg_block_cells = cells;
                    auto vc = [&] { launch_profile_kernel<T>(b, 4, 0, st); };
                    const double ms = in_graph ? time_graph(vc, 3) : time_it(vc, 2);
                    if (cells == def.mg_block_cells) dms += ms;
                    if (ms < best) { best = ms; bc = cells; }
                }
                b.tune.mg_block_cells = bc;
                tms += best;
            }
            double best = 1e30;
            int bs = def.sweep_blocks_per_sm;
            for (int per : {0, 3, 2}) {
                b.tune.sweep_blocks_per_sm = per;
                const double ms = time_it([&] { launch_profile_kernel<T>(b, 3, 0, st); }, 5);
                if (per == def.sweep_blocks_per_sm) dms += ms;
                if (ms < best) { best = ms; bs = per; }
            }
            b.tune.sweep_blocks_per_sm = bs;
            tms += best;
        }
        CKL();
        tune_default_ms = dms;
        tune_tuned_ms = tms;
        tuned = true;
        drop_graphs();   // captured iterations hold the old launch shapes
        {
            std::lock_guard<std::mutex> lk(tune_mu());
            tune_cache()[key] = TuneVal{b.tune, dms, tms};
        }
        return get_tuning(out);
    }
    int get_tuning(suli_tuning *out) override
    {
        if (!out) return SULI_OK;
        out->convdiff_planes = b.tmaps ? CD_PLANES[b.tune.cd_variant] : 0;
        out->mg_block_cells = b.tune.mg_block_cells;
        out->sweep_blocks_per_sm = b.tune.sweep_blocks_per_sm;
        out->tuned = tuned ? 1 : 0;
        out->default_ms = tune_default_ms;
        out->tuned_ms = tune_tuned_ms;
        return SULI_OK;
    }

    // ---- routines -------------------------------------------------------------
    int heaviside_init() override
    {
        density_changed();
        launch_heaviside<T>(b, 1, st);
        CKL();
        return read_scalars();
    }

    int level_set() override
    {
        density_changed();
        int rc;
        if ((rc = setsc(S_DTADV, dt))) return rc;
        if ((rc = setsc(S_RINREPLAY, (double)replay_reinit))) return rc;
        launch_level_set_adv<T>(b, st);
        launch_reinit<T>(b, P[0].reinit_max_iter, st);
        launch_heaviside<T>(b, 0, st);
        CKL();
        if ((rc = read_scalars())) return rc;
        if ((rc = check_finite())) return rc;
        vol_loops = 0;
        for (;;) {
            bool any = false;
            for (int c = 0; c < ncases; ++c) any |= (sc(c, S_VOLACTIVE) != 0.0);
            if (!any) break;
            if (vol_loops >= P[0].vol_loop_max) {
                warn |= (1 << SULI_VOL_LOOP_CAP);
                break;
            }
            launch_volcorr<T>(b, st);
            CKL();
            ++vol_loops;
            if ((rc = read_scalars())) return rc;
        }
        reinit_iters = (int)sc(0, S_RINITER);
        // curv_ls1 after the volume correction (14_level_set.f90:269-270)
        if (any_tens()) {
            launch_curvature<T>(b, st);
            CKL();
        }
        return SULI_OK;
    }

    // a NaN or Inf anywhere in a case's velocity or level set reaches its
    // volume integral (this step's heaviside) or its max|div| (the last
    // conmassa, which counts a NaN divergence as infinite); reads the host
    // mirror of the scalars, so call it after read_scalars()
    int check_finite()
    {
        for (int c = 0; c < ncases; ++c) {
            const double v = sc(c, S_VOLINS), m = sc(c, S_MAXDIV);
            if (sc(c, S_TMAERR) != 0.0)
                return fail(SULI_DEVICE_TIMEOUT, "case " + std::to_string(c) +
                                                     ": a bounded wait for a TMA copy gave up (convdiff)");
            if (!std::isfinite(v) || !std::isfinite(m))
                return fail(SULI_NONFINITE, "case " + std::to_string(c) + ": non-finite state (vol_ins " +
                                                std::to_string(v) + ", max|div| " + std::to_string(m) + ")");
        }
        return SULI_OK;
    }

    bool any_tens() const
    {
        for (const auto &q : P) if (q.t_tens == 1) return true;
        return false;
    }

    bool any_ibm() const
    {
        for (const auto &q : P) if (q.ibm_t == 2) return true;
        return false;
    }
    bool any_inflow() const
    {
        for (const auto &q : P) if (q.ccx0 == 3) return true;
        return false;
    }

    int contorno(int nlock) override
    {
        if (nlock < 1 || nlock > 3) return fail(SULI_BAD_ARG, "nlock must be 1, 2 or 3");
        if (nlock == 3) {
            // level-set IBM (3_contorno.f90:651-659); nothing without an obstacle
            if (!any_ibm()) return SULI_OK;
            density_changed();
            int rc = setsc(S_RINREPLAY, -1.0);
            if (rc) return rc;
            launch_ibm_levelset<T>(b, st);
            if (sizeof(T) == 4) launch_sync_masters<T>(b, st);   // image values -> FP64 level-set master
            launch_reinit<T>(b, P[0].reinit_max_iter, st, 0);
            launch_heaviside<T>(b, -1, st);
            CKL();
            return SULI_OK;
        }
        if (any_ibm()) launch_ibm_velocity<T>(b, st);     // 3_contorno.f90:85-90
        // mixed form: the IBM image values (FP32) into the FP64 masters before
        // the plane fills, which run on both (the inflow writes both)
        if (sizeof(T) == 4) launch_sync_masters<T>(b, st);
        launch_contorno<T>(b, nlock, st, inflow_calls, sg_capturing ? 1 : 0);
        if (any_inflow()) inflow_calls += (nlock == 2) ? 2 : 1;
        if (nlock == 2) launch_outflow_balance<T>(b, st);
        CKL();
        return SULI_OK;
    }

    int ibm_setup() override
    {
        density_changed();
        // obstaculo() for ibm_t = 2 (3_contorno.f90:991-1002): reinitialise the
        // four obstacle level sets, then mark the image points
        for (int t = 1; t <= 4; ++t) launch_reinit<T>(b, P[0].reinit_max_iter, st, t);
        launch_ibm_posicoes<T>(b, st);
        CKL();
        return sync();
    }

    bool any_keq() const
    {
        for (const auto &q : P) if (q.m_turb >= 2) return true;
        return false;
    }
    bool ipa() const { return P[0].t_press == 2 && (P[0].mms_t == 0 || P[0].project_under_mms); }

    int visco() override
    {
        launch_visco<T>(b, any_keq() ? ntt : 0, a_dt, st);
        CKL();
        return SULI_OK;
    }
    int exp_press() override
    {
        if (P[0].t_press != 2) return fail(SULI_BAD_CONFIG, "exp_press belongs to the IPA (t_press = 2)");
        launch_exp_press<T>(b, st);
        CKL();
        return SULI_OK;
    }
    int contorno_les() override
    {
        launch_contorno_les<T>(b, st);
        CKL();
        return SULI_OK;
    }
    bool stored(int icase, int f) override { return dev_ptr(icase, f) != nullptr; }
    bool any_waves() const
    {
        for (const auto &q : P) if (q.wave_t > 0) return true;
        return false;
    }
    int boundary_waves() override
    {
        if (!any_waves()) return SULI_OK;
        launch_waves<T>(b, t, st, sg_capturing ? 1 : 0);
        CKL();
        return SULI_OK;
    }
    int convdiff(int fuse) override
    {
        if (fuse) launch_sponge<T>(b, st);     // complementos' sponge_layer call
        if (b.tmaps) launch_convdiff_tma<T>(b, fuse, st);
        else launch_convdiff<T>(b, fuse, st);
        CKL();
        return SULI_OK;
    }
    int complementos() override
    {
        launch_sponge<T>(b, st);
        launch_complementos<T>(b, st);
        CKL();
        return SULI_OK;
    }
    int tempo() override
    {
        launch_tempo<T>(b, tt, sg_capturing ? -1 : it, st);
        CKL();
        return SULI_OK;
    }
    int set_stage(int tt_) override
    {
        if (tt_ < 1 || tt_ > 3) return fail(SULI_BAD_ARG, "stage must be 1..3");
        tt = tt_;
        dt = a_dt[tt - 1];
        int rc = setsc(S_DT, dt);
        if (rc) return rc;
        return setsc(S_IDT, (dt != 0.0) ? 1.0 / dt : 0.0);
    }

    // CG loop: the persistent tile kernels over the active cases (default), or
    // one thread-block cluster per case for the whole loop (SULI_CG_PATH=clusters)
    int cg_path = -1;   // -1 undecided, 0 tiles, 1 clusters
    bool use_cluster()
    {
        if (cg_path < 0) {
            const char *env = std::getenv("SULI_CG_PATH");
            cg_path = (env && std::string(env) == "clusters" && cluster_cg_size<T>() > 0) ? 1 : 0;
        }
        return cg_path == 1;
    }

    // SULI_CG_TRACE=1: one line per FP64 refinement pass of case 0 on stderr
    static bool cg_trace()
    {
        static const bool on = [] {
            const char *e = std::getenv("SULI_CG_TRACE");
            return e && std::atoi(e) == 1;
        }();
        return on;
    }

    int graddin(int32_t *iters) override
    {
        int rc;
        const int si = (tt >= 1 && tt <= 3) ? tt - 1 : 0;
        if ((rc = setsc(S_CGREPLAY, (double)replay_cg[si]))) return rc;
        const int cgmax = P[0].cg_max_iter;
        int maxit = 0;
        if (sizeof(T) == sizeof(double)) {
            launch_cg_setup<T>(b, st);
            CKL();
            int done = 0;
            int chunk = std::max(1, std::min(prev_cg[si], cgmax));
            if (use_cluster()) {
                if ((rc = ev_begin())) return rc;
                CK(launch_cg_cluster<T>(b, 0, st));
                if ((rc = ev_end())) return rc;
                if ((rc = read_scalars())) return rc;
                chunk = 0;
            }
            int slot = 0;
            if (chunk > 0) launch_cg_table<T>(b, slot, st);
            for (; chunk > 0;) {
                if ((rc = ev_begin())) return rc;
                slot = launch_cg_iters<T>(b, chunk, slot, 0, st);
                CKL();
                if ((rc = ev_end())) return rc;
                done += chunk;
                if ((rc = read_scalars())) return rc;
                bool any = false;
                for (int c = 0; c < ncases; ++c) any |= (sc(c, S_CGACTIVE) != 0.0);
                if (!any || done >= cgmax) break;
                chunk = std::max(4, std::min(64, done / 8));
            }
            launch_cg_finish<T>(b, st);
            CKL();
            for (int c = 0; c < ncases; ++c) maxit = std::max(maxit, (int)sc(c, S_CGITER));
            cg_outer[si] = 0;
        } else {
            const bool mg = b.nlev > 1;
            // SULI_OP_CACHE=0: rebuild the operator in every solve (the
            // reference's order of work; the same bits)
            const char *oc = std::getenv("SULI_OP_CACHE");
            if (oc && std::atoi(oc) == 0) op_valid = false;
            if (!op_valid) {
                launch_cg_refine_operator<T>(b, st);
                if (mg) launch_mg_coarsen<T>(b, st);
                op_valid = true;
            }
            launch_cg_refine_setup<T>(b, st);
            CKL();
            int done = 0;
            int passes = 0;
            for (;;) {
                // FP32 pass until every refining case meets its inner target
                int chunk = mg ? std::max(2, std::min(prev_cg[si], 16)) : std::max(4, std::min(prev_cg[si], 256));
                int pass_done = 0;
                if (!mg && use_cluster()) {
                    if ((rc = ev_begin())) return rc;
                    CK(launch_cg_cluster<T>(b, 1, st));
                    if ((rc = ev_end())) return rc;
                    chunk = 0;
                }
                int slot = 0;
                if (chunk > 0) {
                    launch_cg_table<T>(b, slot, st);
                    if (mg) launch_pcg_start<T>(b, slot, st);
                }
                for (; chunk > 0;) {
                    if ((rc = ev_begin())) return rc;
                    slot = mg ? pcg_iters(chunk, slot) : launch_cg_iters<T>(b, chunk, slot, 1, st);
                    if (slot < 0) return fail(SULI_CUDA_ERROR, "launching the CG iteration graph failed");
                    CKL();
                    if ((rc = ev_end())) return rc;
                    done += chunk;
                    pass_done += chunk;
                    if ((rc = read_scalars())) return rc;
                    bool any = false;
                    for (int c = 0; c < ncases; ++c) any |= (sc(c, S_CGACTIVE) != 0.0);
                    if (!any || done >= cgmax + 256) break;
                    chunk = mg ? std::max(2, std::min(8, pass_done / 2)) : std::max(4, std::min(64, pass_done / 4));
                }
                launch_cg_refine_next<T>(b, st);
                CKL();
                if ((rc = read_scalars())) return rc;
                if (cg_trace())
                    std::fprintf(stderr, "suli cg trace: stage %d pass %d iterations %d fp64 r.r %.3e threshold %.3e fp32 r.r %.3e\n",
                                 tt, (int)std::fabs(sc(0, S_OUTER)), pass_done, sc(0, S_RRTRUE), sc(0, S_THR), sc(0, S_RR));
                bool all = true;
                passes = 0;
                for (int c = 0; c < ncases; ++c) {
                    all &= (sc(c, S_OUTER) < 0.0);
                    passes = std::max(passes, (int)std::fabs(sc(c, S_OUTER)));
                }
                if (all || done >= cgmax + 256) break;
            }
            launch_cg_refine_finish<T>(b, st);
            CKL();
            for (int c = 0; c < ncases; ++c) {
                maxit = std::max(maxit, (int)sc(c, S_CGITER));
                if (sc(c, S_STALLED) != 0.0) warn |= (1 << SULI_CG_STALLED);
            }
            cg_outer[si] = passes;
        }
        if (prof)
            for (int c = 0; c < ncases; ++c) cg_cell_iters += cells(c) * sc(c, S_CGITER);
        cg_iters[si] = maxit;
        // (the mixed form's r.r is the unit operator's: the stage's over dt)
        cg_res[si] = (sizeof(T) == sizeof(double)) ? sc(0, S_RR) : sc(0, S_RRTRUE) * dt;
        prev_cg[si] = std::max(1, sizeof(T) == sizeof(double) ? maxit : maxit / std::max(1, cg_outer[si]));
        if (iters) *iters = maxit;
        if (maxit >= cgmax && replay_cg[si] < 0) {
            warn |= (1 << SULI_CG_MAXITER);
            return fail(SULI_CG_MAXITER, "CG reached cg_max_iter (\"pulou pressao\")");
        }
        return SULI_OK;
    }

    int posdin() override
    {
        if (P[0].t_press != 1)
            return fail(SULI_BAD_CONFIG, "posdin projects for t_press = 1 only (the IPA step has no posdin)");
        launch_posdin<T>(b, st);
        CKL();
        for (int c = 0; c < ncases; ++c)
            CK(cudaMemcpyAsync(hc[c].prd, hc[c].prd1, sizeof(T) * (size_t)hc[c].g.total, cudaMemcpyDeviceToDevice, st));
        return SULI_OK;
    }

    int conmassa(double *maxdiv) override
    {
        launch_conmassa<T>(b, st);
        CKL();
        if (maxdiv) {
            int rc = read_scalars();
            if (rc) return rc;
            *maxdiv = sc(0, S_MAXDIV);
            if ((rc = check_finite())) return rc;
        }
        return SULI_OK;
    }

    int mms_error(double *err) override
    {
        launch_mms_error<T>(b, st);
        CKL();
        int rc = read_scalars();
        if (rc) return rc;
        for (int q = 0; q < 4; ++q) err[q] = sc(0, S_ERR0 + q);
        return SULI_OK;
    }

    // the body of the time loop, 1_principal.f90:69-124 (PLOT output excluded)
    int step(int n) override
    {
        int rc;
        for (int s = 0; s < n; ++s) {
            if (step_graph_state >= 0 && step_graph_eligible()) {
                rc = step_by_graph();
                if (rc == 0) { step_graph_state = 1; continue; }
                if (rc > 0) return rc;
                step_graph_state = -1;    // the graph could not be built: the host-driven step
            }
            it = it + 1;
            t = t + dt;
            if ((rc = level_set())) return rc;
            if ((rc = contorno(3))) return rc;
            if (ipa() && (rc = exp_press())) return rc;          // 1_principal.f90:82
            if ((rc = visco())) return rc;
            for (int q = 1; q <= ntt; ++q) {
                if ((rc = set_stage(q))) return rc;
                if ((rc = convdiff(1))) return rc;
                if ((rc = tempo())) return rc;
                if ((rc = boundary_waves())) return rc;          // wave_t > 0, :93
                if ((rc = contorno(2))) return rc;
                if (P[0].mms_t == 0 || P[0].project_under_mms) {
                    if (P[0].t_press == 1) {
                        rc = graddin(nullptr);
                        if (rc && rc != SULI_CG_MAXITER) return rc;
                        if ((rc = posdin())) return rc;
                    }
                    if ((rc = contorno(1))) return rc;
                }
            }
            if (ipa()) {                                          // :111, no posdin
                rc = graddin(nullptr);
                if (rc && rc != SULI_CG_MAXITER) return rc;
            }
            if ((rc = conmassa(nullptr))) return rc;
            // the autotuner, once, after the handle's first step
            if (!tuned && tune_env == 1 && (rc = autotune(nullptr))) return rc;
        }
        // a TMA wait that gave up in the last step (the check in level_set
        // covers the steps before it)
        if (n > 0) {
            if ((rc = read_scalars())) return rc;
            if ((rc = check_finite())) return rc;
        }
        return SULI_OK;
    }
};

// ---------------------------------------------------------------------------
static int check_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(SULI_NO_DEVICE, std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count 0"));
    return SULI_OK;
}

extern "C" int suli_create_batch(const suli_params *p, int ncases, suli_handle **out)
{
    if (!p || !out || ncases < 1) return fail(SULI_BAD_ARG, "bad arguments to suli_create_batch");
    *out = nullptr;
    for (int c = 0; c < ncases; ++c) {
        int rc = validate(p[c]);
        if (rc) return rc;
        if (p[c].precision != p[0].precision || p[c].t_tempo != p[0].t_tempo || p[c].mms_t != p[0].mms_t ||
            p[c].dt != p[0].dt || p[c].reinit_max_iter != p[0].reinit_max_iter ||
            p[c].project_under_mms != p[0].project_under_mms || p[c].t_press != p[0].t_press)
            return fail(SULI_BAD_CONFIG, "cases of a batch must share precision, t_tempo, mms_t, t_press, dt and reinit_max_iter");
    }
    int rc = check_device();
    if (rc) return rc;
    ImplBase *impl;
    if (p[0].precision == SULI_PREC_FP64) {
        auto *im = new Impl<double>();
        rc = im->create(p, ncases);
        impl = im;
    } else {
        auto *im = new Impl<float>();
        rc = im->create(p, ncases);
        impl = im;
    }
    if (rc) {
        delete impl;
        return rc;
    }
    *out = new suli_handle{impl};
    return SULI_OK;
}

extern "C" int suli_create(const suli_params *p, suli_handle **out) { return suli_create_batch(p, 1, out); }

extern "C" int suli_num_cases(const suli_handle *h, int *n)
{
    if (!h || !n) return fail(SULI_BAD_ARG, "null argument");
    *n = h->impl->ncases;
    return SULI_OK;
}

extern "C" int suli_destroy(suli_handle *h)
{
    if (!h) return SULI_OK;
    delete h->impl;
    delete h;
    return SULI_OK;
}

#define HCHK()                                                   \
    do {                                                         \
        if (!h) return fail(SULI_BAD_ARG, "null handle");        \
    } while (0)

extern "C" int suli_upload_field(suli_handle *h, int icase, int field, const void *host)
{
    HCHK();
    if (!host) return fail(SULI_BAD_ARG, "null host pointer");
    return h->impl->copy_field(icase, field, const_cast<void *>(host), true);
}

extern "C" int suli_download_field(suli_handle *h, int icase, int field, void *host)
{
    HCHK();
    if (!host) return fail(SULI_BAD_ARG, "null host pointer");
    return h->impl->copy_field(icase, field, host, false);
}

extern "C" int suli_upload_fields(suli_handle *h, int n, const int32_t *cases, const int32_t *fields,
                                  const void *const *host)
{
    HCHK();
    return h->impl->copy_fields(n, cases, fields, const_cast<void *const *>(host), true);
}

extern "C" int suli_download_fields(suli_handle *h, int n, const int32_t *cases, const int32_t *fields,
                                    void *const *host)
{
    HCHK();
    return h->impl->copy_fields(n, cases, fields, host, false);
}

extern "C" int suli_set_scalar(suli_handle *h, int icase, int s, double v)
{
    HCHK();
    ImplBase *im = h->impl;
    switch (s) {
    case SULI_S_T: im->t = v; return SULI_OK;
    case SULI_S_DT: im->dt = v; return SULI_OK;
    case SULI_S_IT: im->it = (int)v; return SULI_OK;
    case SULI_S_TT: im->tt = (int)v; return SULI_OK;
    case SULI_S_RNG: im->inflow_calls = (unsigned long long)v; return SULI_OK;
    case SULI_S_VOL_INI:
    case SULI_S_VOL_INS: {
        if (icase < 0 || icase >= im->ncases) return fail(SULI_BAD_ARG, "case index out of range");
        return im->write_case_scalar(icase, s == SULI_S_VOL_INI ? S_VOLINI : S_VOLINS, v);
    }
    default: return fail(SULI_BAD_ARG, "scalar not settable");
    }
}

extern "C" int suli_get_scalar(suli_handle *h, int icase, int s, double *v)
{
    HCHK();
    if (!v) return fail(SULI_BAD_ARG, "null pointer");
    ImplBase *im = h->impl;
    if (icase < 0 || icase >= im->ncases) return fail(SULI_BAD_ARG, "case index out of range");
    switch (s) {
    case SULI_S_T: *v = im->t; return SULI_OK;
    case SULI_S_DT: *v = im->dt; return SULI_OK;
    case SULI_S_IT: *v = im->it; return SULI_OK;
    case SULI_S_TT: *v = im->tt; return SULI_OK;
    case SULI_S_RNG: *v = (double)im->inflow_calls; return SULI_OK;
    default: break;
    }
    int rc = im->read_scalars();
    if (rc) return rc;
    const double *sc = im->hsc + (size_t)icase * S_NSCAL;
    switch (s) {
    case SULI_S_VOL_INI: *v = sc[S_VOLINI]; return SULI_OK;
    case SULI_S_VOL_INS: *v = sc[S_VOLINS]; return SULI_OK;
    case SULI_S_MAXDIV: *v = sc[S_MAXDIV]; return SULI_OK;
    default: return fail(SULI_BAD_ARG, "unknown scalar");
    }
}

extern "C" int suli_set_replay(suli_handle *h, const int32_t cg[3], int32_t reinit)
{
    HCHK();
    for (int q = 0; q < 3; ++q) h->impl->replay_cg[q] = cg ? cg[q] : -1;
    h->impl->replay_reinit = reinit;
    return SULI_OK;
}

extern "C" int suli_heaviside_init(suli_handle *h) { HCHK(); return h->impl->heaviside_init(); }
extern "C" int suli_ibm_setup(suli_handle *h) { HCHK(); return h->impl->ibm_setup(); }
extern "C" int suli_level_set(suli_handle *h) { HCHK(); return h->impl->level_set(); }
extern "C" int suli_contorno(suli_handle *h, int nlock) { HCHK(); return h->impl->contorno(nlock); }
extern "C" int suli_visco(suli_handle *h) { HCHK(); return h->impl->visco(); }
extern "C" int suli_convdiff(suli_handle *h) { HCHK(); return h->impl->convdiff(0); }
extern "C" int suli_complementos(suli_handle *h) { HCHK(); return h->impl->complementos(); }
extern "C" int suli_tempo(suli_handle *h) { HCHK(); return h->impl->tempo(); }
extern "C" int suli_graddin(suli_handle *h, int32_t *iters) { HCHK(); return h->impl->graddin(iters); }
extern "C" int suli_posdin(suli_handle *h) { HCHK(); return h->impl->posdin(); }
extern "C" int suli_exp_press(suli_handle *h) { HCHK(); return h->impl->exp_press(); }
extern "C" int suli_contorno_les(suli_handle *h) { HCHK(); return h->impl->contorno_les(); }
extern "C" int suli_boundary_waves(suli_handle *h) { HCHK(); return h->impl->boundary_waves(); }
extern "C" int suli_conmassa(suli_handle *h, double *m) { HCHK(); return h->impl->conmassa(m); }
extern "C" int suli_mms_error(suli_handle *h, double err[4])
{
    HCHK();
    if (!err) return fail(SULI_BAD_ARG, "null pointer");
    return h->impl->mms_error(err);
}
extern "C" int suli_set_stage(suli_handle *h, int tt) { HCHK(); return h->impl->set_stage(tt); }
extern "C" int suli_step(suli_handle *h, int n)
{
    HCHK();
    if (n < 0) return fail(SULI_BAD_ARG, "nsteps < 0");
    return h->impl->step(n);
}
extern "C" int suli_synchronize(suli_handle *h) { HCHK(); return h->impl->sync(); }

extern "C" int suli_diagnostics(suli_handle *h, int icase, suli_diag *d)
{
    HCHK();
    if (!d) return fail(SULI_BAD_ARG, "null pointer");
    ImplBase *im = h->impl;
    if (icase < 0 || icase >= im->ncases) return fail(SULI_BAD_ARG, "case index out of range");
    int rc = im->read_scalars();
    if (rc) return rc;
    const double *sc = im->hsc + (size_t)icase * S_NSCAL;
    std::memset(d, 0, sizeof(*d));
    d->vol_ini = sc[S_VOLINI];
    d->vol_ins = sc[S_VOLINS];
    d->maxdiv = sc[S_MAXDIV];
    d->t = im->t;
    for (int q = 0; q < 3; ++q) {
        d->cg_iters[q] = im->cg_iters[q];
        d->cg_outer[q] = im->cg_outer[q];
        d->cg_res[q] = im->cg_res[q];
    }
    d->reinit_iters = (int)sc[S_RINITER];
    d->vol_loops = im->vol_loops;
    d->it = im->it;
    d->status_flags = im->warn;
    im->warn = 0;
    return SULI_OK;
}

extern "C" int suli_autotune(suli_handle *h, suli_tuning *out) { HCHK(); return h->impl->autotune(out); }
extern "C" int suli_get_tuning(suli_handle *h, suli_tuning *out) { HCHK(); return h->impl->get_tuning(out); }

extern "C" int suli_get_stream(suli_handle *h, void **stream)
{
    HCHK();
    if (!stream) return fail(SULI_BAD_ARG, "null pointer");
    *stream = h->impl->stream();
    return SULI_OK;
}

extern "C" int suli_profile(suli_handle *h, int enable)
{
    HCHK();
    ImplBase *im = h->impl;
    im->prof = (enable != 0);
    im->launch0 = g_launches.load();
    im->cg_ms = 0.0;
    im->cg_cell_iters = 0.0;
    return SULI_OK;
}

extern "C" int suli_profile_read(suli_handle *h, suli_profile_t *out)
{
    HCHK();
    if (!out) return fail(SULI_BAD_ARG, "null pointer");
    ImplBase *im = h->impl;
    out->launches = g_launches.load() - im->launch0;
    out->cg_ms = im->cg_ms;
    out->cg_cell_iters = im->cg_cell_iters;
    // bytes the three iteration kernels move per cell: A reads p and the three
    // scaled coefficients and writes mp; B reads e, p, r, mp and writes e, r;
    // C reads r, p and writes p -- 14 arrays of the storage type
    out->cg_bytes_per_cell_iter = 14.0 * (im->P[0].precision == SULI_PREC_FP64 ? 8.0 : 4.0);
    return SULI_OK;
}

extern "C" int suli_time_kernel(suli_handle *h, int kernel, int reps, double *ms_per_launch,
                                double *bytes_per_launch)
{
    HCHK();
    if (!ms_per_launch || !bytes_per_launch) return fail(SULI_BAD_ARG, "null pointer");
    return h->impl->time_kernel(kernel, reps, ms_per_launch, bytes_per_launch);
}

extern "C" int suli_write_fields(suli_handle *h, int icase, const char *path, int t_plot)
{
    HCHK();
    return h->impl->write_fields(icase, path, t_plot);
}

// ---- restart: a binary replacement of restart_salva / restart_ini
// (11_diversos.f90:500-599), which write every state array as formatted text
// and, on reading, reset t and it to zero.  The file holds, little-endian:
// "SULIRST1", int32 version (1), int32 cases, int32 field count, double t,
// int64 it, double dt, uint64 inflow draws, int32 stage; per case int32
// nx, ny, nz, double vol_ini, vol_ins; per case and field int32 id, int64
// count, then the values in the reference layout (double; int32 for the IBM
// masks).  Loading restores the fields, t, it, dt and the counters, so the
// run continues exactly where it was saved.
static const char kRestartMagic[8] = {'S', 'U', 'L', 'I', 'R', 'S', 'T', '1'};

static long long field_count(const suli_params &p, int f)
{
    int lo[3], hi[3];
    if (suli_field_shape(&p, f, lo, hi) != SULI_OK) return -1;
    long long n = 1;
    for (int d = 0; d < 3; ++d) n *= (long long)(hi[d] - lo[d] + 1);
    return n;
}

// every field of case c through one batched transfer (up: host -> device)
static int restart_fields(ImplBase *im, int c, std::vector<std::vector<double>> &dv,
                          std::vector<std::vector<int32_t>> &iv, bool up)
{
    std::vector<int32_t> cases, fields;
    std::vector<void *> hosts;
    dv.resize(SULI_F_COUNT);
    iv.resize(SULI_F_COUNT);
    for (int f = 0; f < SULI_F_COUNT; ++f) {
        // fields of a model the case does not run (k equation, IPA) are not
        // stored: an empty record
        if (!im->stored(c, f)) continue;
        const long long n = field_count(im->P[c], f);
        if (n < 0) return fail(SULI_BAD_ARG, "field shape");
        if (is_int_field(f)) {
            iv[f].resize((size_t)n);
            hosts.push_back(iv[f].data());
        } else {
            dv[f].resize((size_t)n);
            hosts.push_back(dv[f].data());
        }
        cases.push_back(c);
        fields.push_back(f);
    }
    if (up) return SULI_OK;    // the caller fills the buffers, then transfers
    return im->copy_fields((int)fields.size(), cases.data(), fields.data(), hosts.data(), false);
}

extern "C" int suli_restart_save(suli_handle *h, const char *path)
{
    HCHK();
    ImplBase *im = h->impl;
    if (!path) return fail(SULI_BAD_ARG, "null path");
    int rc = im->read_scalars();
    if (rc) return rc;
    std::FILE *fp = std::fopen(path, "wb");
    if (!fp) return fail(SULI_BAD_ARG, std::string("cannot open ") + path);
    bool ok = true;
    auto put = [&](const void *p, size_t n) { ok = ok && std::fwrite(p, 1, n, fp) == n; };
    const int32_t version = 1, nc = im->ncases, nf = SULI_F_COUNT, tt = im->tt;
    const int64_t it = im->it;
    const uint64_t draws = im->inflow_calls;
    put(kRestartMagic, 8); put(&version, 4); put(&nc, 4); put(&nf, 4);
    put(&im->t, 8); put(&it, 8); put(&im->dt, 8); put(&draws, 8); put(&tt, 4);
    for (int c = 0; c < nc; ++c) {
        const int32_t d[3] = {im->P[c].nx, im->P[c].ny, im->P[c].nz};
        const double *sc = im->hsc + (size_t)c * S_NSCAL;
        put(d, 12); put(&sc[S_VOLINI], 8); put(&sc[S_VOLINS], 8);
    }
    for (int c = 0; c < nc && ok; ++c) {
        std::vector<std::vector<double>> dv;
        std::vector<std::vector<int32_t>> iv;
        rc = restart_fields(im, c, dv, iv, false);
        if (rc) { std::fclose(fp); return rc; }
        for (int f = 0; f < SULI_F_COUNT; ++f) {
            const int32_t id = f;
            const int64_t n = is_int_field(f) ? (int64_t)iv[f].size() : (int64_t)dv[f].size();
            put(&id, 4); put(&n, 8);
            if (is_int_field(f)) put(iv[f].data(), (size_t)n * 4);
            else put(dv[f].data(), (size_t)n * 8);
        }
    }
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) return fail(SULI_BAD_ARG, std::string("writing ") + path + " failed");
    return SULI_OK;
}

extern "C" int suli_restart_load(suli_handle *h, const char *path)
{
    HCHK();
    ImplBase *im = h->impl;
    if (!path) return fail(SULI_BAD_ARG, "null path");
    std::FILE *fp = std::fopen(path, "rb");
    if (!fp) return fail(SULI_BAD_ARG, std::string("cannot open ") + path);
    bool ok = true;
    auto get = [&](void *p, size_t n) { ok = ok && std::fread(p, 1, n, fp) == n; };
    auto bad = [&](const std::string &why) { std::fclose(fp); return fail(SULI_BAD_CONFIG, path + std::string(": ") + why); };
    char magic[8];
    int32_t version = 0, nc = 0, nf = 0, tt = 1;
    int64_t it = 0;
    uint64_t draws = 0;
    double t = 0.0, dt = 0.0;
    get(magic, 8); get(&version, 4); get(&nc, 4); get(&nf, 4);
    if (!ok || std::memcmp(magic, kRestartMagic, 8) != 0 || version != 1) return bad("not a restart file of this library");
    if (nc != im->ncases || nf != SULI_F_COUNT) return bad("written for another batch");
    get(&t, 8); get(&it, 8); get(&dt, 8); get(&draws, 8); get(&tt, 4);
    std::vector<double> vini(nc), vins(nc);
    for (int c = 0; c < nc; ++c) {
        int32_t d[3];
        get(d, 12); get(&vini[c], 8); get(&vins[c], 8);
        if (ok && (d[0] != im->P[c].nx || d[1] != im->P[c].ny || d[2] != im->P[c].nz))
            return bad("case " + std::to_string(c) + " has other dimensions");
    }
    if (!ok) return bad("truncated restart file");
    // first pass over the record headers: every record present with the
    // expected id and length and the file long enough, before anything is
    // uploaded (a refused file leaves the handle as it was)
    const long data0 = std::ftell(fp);
    if (data0 < 0 || std::fseek(fp, 0, SEEK_END) != 0) return bad("cannot seek");
    const long long fsize = (long long)std::ftell(fp);
    long long pos = data0;
    for (int c = 0; c < nc; ++c)
        for (int f = 0; f < SULI_F_COUNT; ++f) {
            int32_t id = -1;
            int64_t n = -1;
            if (pos + 12 > fsize || std::fseek(fp, (long)pos, SEEK_SET) != 0) return bad("truncated restart file");
            get(&id, 4); get(&n, 8);
            const int64_t want = im->stored(c, f) ? field_count(im->P[c], f) : 0;
            if (!ok || id != f || n != want) return bad("field " + std::to_string(f) + " of case " + std::to_string(c));
            pos += 12 + n * (is_int_field(f) ? 4 : 8);
            if (pos > fsize) return bad("truncated restart file");
        }
    if (std::fseek(fp, data0, SEEK_SET) != 0) return bad("cannot seek");
    for (int c = 0; c < nc && ok; ++c) {
        std::vector<std::vector<double>> dv;
        std::vector<std::vector<int32_t>> iv;
        int rc = restart_fields(im, c, dv, iv, true);
        if (rc) { std::fclose(fp); return rc; }
        std::vector<int32_t> cases, fields;
        std::vector<void *> hosts;
        for (int f = 0; f < SULI_F_COUNT && ok; ++f) {
            int32_t id = -1;
            int64_t n = -1;
            get(&id, 4); get(&n, 8);
            const int64_t want = is_int_field(f) ? (int64_t)iv[f].size() : (int64_t)dv[f].size();
            if (!ok || id != f || n != want) return bad("field " + std::to_string(f) + " of case " + std::to_string(c));
            if (n == 0) continue;
            if (is_int_field(f)) { get(iv[f].data(), (size_t)n * 4); hosts.push_back(iv[f].data()); }
            else { get(dv[f].data(), (size_t)n * 8); hosts.push_back(dv[f].data()); }
            cases.push_back(c);
            fields.push_back(f);
        }
        if (!ok) break;
        rc = im->copy_fields((int)fields.size(), cases.data(), fields.data(), hosts.data(), true);
        if (rc) { std::fclose(fp); return rc; }
    }
    std::fclose(fp);
    if (!ok) return fail(SULI_BAD_CONFIG, std::string(path) + ": truncated restart file");
    im->t = t;
    im->it = (int)it;
    im->dt = dt;
    im->inflow_calls = draws;
    im->tt = tt;
    for (int c = 0; c < nc; ++c) {
        int rc = im->write_case_scalar(c, S_VOLINI, vini[c]);
        if (!rc) rc = im->write_case_scalar(c, S_VOLINS, vins[c]);
        if (rc) return rc;
    }
    return SULI_OK;
}

extern "C" int suli_last_error(char *buf, size_t len)
{
    if (!buf || len == 0) return SULI_BAD_ARG;
    std::snprintf(buf, len, "%s", g_err.c_str());
    return SULI_OK;
}

extern "C" int suli_device_info(int *sm_count, char *name, size_t name_len)
{
    int rc = check_device();
    if (rc) return rc;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, dev));
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (name && name_len) std::snprintf(name, name_len, "%s", prop.name);
    return SULI_OK;
}
