// suli_kernels.cuh -- launch interface between the C ABI layer and the
// kernel translation units.
#pragma once

#include "suli_common.cuh"

#include <atomic>

namespace suli {

// grid of a persistent kernel: every SM filled to the kernel's own occupancy
// (256 threads per block)
inline int occupancy_grid(const void *fn, size_t dyn_smem = 0)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, dyn_smem);
    return (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
}

// kernels launched by this library (all handles); read by suli_profile_read
extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Launch shapes that the autotuner picks per device and workload shape; every
// choice gives the same bits (only the partition of the work changes).
constexpr int CD_PLANES[3] = {8, 16, 32};   // planes per unit of the TMA-staged convdiff
struct Tuning {
    int cd_variant = 1;           // index into CD_PLANES
    int mg_block_cells = 16384;   // largest level (cells) of the one-block coarse end of the V-cycle; 0: none
    int sweep_blocks_per_sm = 0;  // blocks per SM of the one-pass multigrid sweep; 0: its occupancy limit
};

// A batch of cases with a device copy of their CaseDev table.
template <typename T>
struct Batch {
    CaseDev<T> *dcases = nullptr;     // device table
    CaseDev<T> *hcases = nullptr;     // host mirror
    int ncases = 0;
    int total_tiles = 0;
    int total_units = 0;              // column units of the case grids (all cases)
    int max_plane = 0;                // largest boundary plane (elements)
    double *drk = nullptr;            // TVD-RK3 coefficients a[3], b[3], g[3]
    int *act = nullptr;               // two active-case tables of the CG iteration
    unsigned *act_done = nullptr;     // cases done with the current B phase
    int nlev = 1;                     // grid levels in the tables (multigrid levels, or 1)
    int mg_tiles[MG_MAXL] = {0};      // tiles of multigrid level l over all cases
    const CUtensorMap *tmaps = nullptr;   // per case the tensor maps of the convdiff operands (or null)
    int test_shortfall = 0;           // failure-path test hook of the staged convdiff (SULI_TEST_TMA_SHORTFALL=1)
    int total_cd_units[3] = {0, 0, 0};   // units of the TMA-staged convdiff over all cases, per unit height
    Tuning tune;                      // the autotuner's launch shapes
    long long total_cd_shell = 0;     // boundary-shell positions of convdiff over all cases
    dim3 block() const { return dim3(TX, TY, TZ); }
    dim3 cblock() const { return dim3(COL_X, COL_Y, 1); }   // persistent (column) kernels
};

// level set (k_levelset.cu)
template <typename T> void launch_level_set_adv(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_reinit(const Batch<T> &b, int max_iter, cudaStream_t s, int target = 0);
template <typename T> void launch_heaviside(const Batch<T> &b, int set_ini, cudaStream_t s);
template <typename T> void launch_curvature(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_volcorr(const Batch<T> &b, cudaStream_t s);

// momentum (k_momentum.cu)
// visco; keq_stages > 0 runs the k equation's sub-stages (a_dt[0..]) for the
// m_turb >= 2 cases between the strain and the face viscosities
template <typename T> void launch_visco(const Batch<T> &b, int keq_stages, const double *a_dt, cudaStream_t s);
// k equation and IPA (k_keq.cu)
template <typename T> void launch_keq(const Batch<T> &b, int ntt, const double *a_dt, cudaStream_t s);
template <typename T> void launch_contorno_les(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_exp_press(const Batch<T> &b, cudaStream_t s);
// (tdev: the time from case 0's S_TIME instead of t, for the step graph)
template <typename T> void launch_waves(const Batch<T> &b, double t, cudaStream_t s, int tdev = 0);
template <typename T> void launch_convdiff(const Batch<T> &b, int fuse_compl, cudaStream_t s);
// convdiff (+ complementos) with its operands staged by TMA tensor loads
// (k_convdiff_tma.cu): b.tmaps holds 8 maps per case (u, v, w, rho, mu, xmu,
// ymu, zmu: each the case's padded box, box 40 x 12 x 1)
template <typename T> void launch_convdiff_tma(const Batch<T> &b, int fuse_compl, cudaStream_t s);
int convdiff_units(int nx, int ny, int nz, int variant);
long long convdiff_shell_positions(int nx, int ny, int nz);
constexpr int CD_MAP_BOX_X = 40, CD_MAP_BOX_Y = 12;
// sponge_layer's epis_z for the esp_type > 0 cases (before complementos)
template <typename T> void launch_sponge(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_complementos(const Batch<T> &b, cudaStream_t s);
// (it < 0: the step number from case 0's S_ITSTEP, for the step graph)
template <typename T> void launch_tempo(const Batch<T> &b, int tt, int it, cudaStream_t s);
template <typename T> void launch_posdin(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_conmassa(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_mms_error(const Batch<T> &b, cudaStream_t s);

// boundary conditions (k_bc.cu)
// (cdev: the inflow's call count is case 0's S_RNGBASE plus rng_call, for the step graph)
template <typename T> void launch_contorno(const Batch<T> &b, int nlock, cudaStream_t s, unsigned long long rng_call = 0,
                                           int cdev = 0);
// balanced free outflow (outflow_flux = 1, ccxf = 4): after contorno(2), on the
// FP64 masters where the mixed form has them, then their FP32 copies
template <typename T> void launch_outflow_balance(const Batch<T> &b, cudaStream_t s);
// mixed form: FP32 velocity and level-set values the IBM images wrote -> FP64 masters
template <typename T> void launch_sync_masters(const Batch<T> &b, cudaStream_t s);

// immersed boundary (k_ibm.cu)
template <typename T> void launch_ibm_posicoes(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_ibm_velocity(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_ibm_levelset(const Batch<T> &b, cudaStream_t s);

// pressure (k_cg.cu)
template <typename T> void launch_cg_setup(const Batch<T> &b, cudaStream_t s);
// active-case table `slot` := cases with S_CGACTIVE set
template <typename T> void launch_cg_table(const Batch<T> &b, int slot, cudaStream_t s);
// n iterations from table `slot` (mode 0: the case's stop rule, 1: one FP32
// pass of the mixed form); returns the slot of the table now current
template <typename T> int launch_cg_iters(const Batch<T> &b, int n, int slot, int mode, cudaStream_t s);
// mixed form, multigrid-preconditioned passes: start (z = M r, p = z) and n
// iterations from table `slot` (returns the current slot)
template <typename T> void launch_pcg_start(const Batch<T> &b, int slot, cudaStream_t s);
template <typename T> int launch_pcg_iters(const Batch<T> &b, int n, int slot, cudaStream_t s);

// profiling: one launch of kernel `kernel` over every case (table slot 2;
// prepare != 0 builds that table first); returns -1 for an unknown kernel
template <typename T> int launch_profile_kernel(const Batch<T> &b, int kernel, int prepare, cudaStream_t s);
template <typename T> int launch_mg_smooth0(const Batch<T> &b, const int *tab, int grid, cudaStream_t s);
template <typename T> int launch_mg_sweep0(const Batch<T> &b, const int *tab, cudaStream_t s);
template <typename T> int launch_mg_vcycle_prof(const Batch<T> &b, const int *tab, cudaStream_t s);

// multigrid (k_mg.cu): coarse operators from level 0, one V-cycle over a table
template <typename T> void launch_mg_coarsen(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_mg_vcycle(const Batch<T> &b, const int *tab, int grid, cudaStream_t s);
template <typename T> void launch_cg_finish(const Batch<T> &b, cudaStream_t s);
// mixed form: FP64 residual recomputation and correction around the FP32 inner CG
// field output (k_output.cu)
template <typename T> void launch_prtscr(const Batch<T> &b, int icase, float *out, int t_plot, cudaStream_t s);
template <typename T> void launch_cg_refine_operator(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_cg_refine_setup(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_cg_refine_next(const Batch<T> &b, cudaStream_t s);
template <typename T> void launch_cg_refine_finish(const Batch<T> &b, cudaStream_t s);

// CG loop of batched small cases, one thread-block cluster per case (k_cg_cluster.cu)
template <typename T> cudaError_t launch_cg_cluster(const Batch<T> &b, int mode, cudaStream_t s);
template <typename T> int cluster_cg_size();

// per-case scalar kernels
template <typename T> void launch_set_scalar(const Batch<T> &b, int slot, double v, cudaStream_t s);
// whole-step graph (k_stepgraph.cu): the condition of a device loop (mode 0:
// any S_CGACTIVE, 1: any S_OUTER >= 0, 2: any S_VOLACTIVE; trip counter
// slot `trip` of case 0 below cap), a stage's solve statistics, the reset
// of the counters at the start of the step
template <typename T> void launch_loop_cond(const Batch<T> &b, int mode, int trip, double cap,
                                            cudaGraphConditionalHandle h, cudaStream_t s);
template <typename T> void launch_stage_record(const Batch<T> &b, int si, cudaStream_t s);
template <typename T> void launch_step_reset(const Batch<T> &b, cudaStream_t s);

}  // namespace suli
