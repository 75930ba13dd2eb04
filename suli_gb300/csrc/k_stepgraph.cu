// k_stepgraph.cu -- device-side loop control of the whole-step CUDA graph
// (mixed form): the loops of the time step that the host drove by reading
// the per-case scalars -- the FP64 refinement passes of graddin
// (9_grad.f90:398-587 in the reference's Jacobi form), the FP32 CG
// iterations inside a pass, the volume-correction loop of level_set
// (14_level_set.f90:243) -- become conditional WHILE nodes whose condition
// a one-block kernel sets from the same scalars.
//
// Every loop is bounded on the device as well: a trip counter kept in case
// 0's scalars stops the loop at its cap even if the scalars never clear (a
// NaN state, say), so a graph launch always ends.  The counters are also
// how the host learns the trip counts after the step (launch accounting,
// diagnostics).
#include "suli_kernels.cuh"

namespace suli {

// condition of loop `mode` (0: a case's FP32 CG iterates, S_CGACTIVE; 1: a
// case still refines, S_OUTER >= 0; 2: a case's volume correction runs,
// S_VOLACTIVE) and the trip counter cs[0].sc[trip] below cap; counts the
// trip when it sets the condition
template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_loop_cond(const CaseDev<T> *__restrict__ cs, int N, int mode, int trip,
                                                        double cap, cudaGraphConditionalHandle h)
{
    int any = 0;
    for (int c = tid_lin(); c < N; c += NTHREADS) {
        const double *s = cs[c].sc;
        if (mode == 0) any |= (__ldcg(&s[S_CGACTIVE]) != 0.0);
        else if (mode == 1) any |= (__ldcg(&s[S_OUTER]) >= 0.0);
        else any |= (__ldcg(&s[S_VOLACTIVE]) != 0.0);
    }
    any = __syncthreads_or(any);
    if (tid_lin() == 0) {
        double *t = cs[0].sc + trip;
        const bool go = any && *t < cap;
        if (go) *t = *t + 1.0;
        cudaGraphSetConditional(h, go ? 1u : 0u);
    }
}

// a stage's solve statistics into the per-case stage slots (graddin of
// stage si): iterations, FP64 passes, stagnation
template <typename T>
__global__ void k_stage_record(const CaseDev<T> *__restrict__ cs, int N, int si)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    double *s = cs[c].sc;
    s[S_STIT0 + si] = s[S_CGITER];
    s[S_STOUT0 + si] = fabs(s[S_OUTER]);
    if (s[S_STALLED] != 0.0) s[S_STSTALL] = 1.0;
}

// the trip counters and the stagnation flag at the start of a step graph
template <typename T>
__global__ void k_step_reset(const CaseDev<T> *__restrict__ cs, int N)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    double *s = cs[c].sc;
    s[S_STSTALL] = 0.0;
    if (c == 0)
        for (int q = S_TRIP_VOL; q <= S_TRIP_IN2; ++q) s[q] = 0.0;
}

template <typename T>
void launch_loop_cond(const Batch<T> &b, int mode, int trip, double cap, cudaGraphConditionalHandle h, cudaStream_t s)
{
    k_loop_cond<T><<<1, NTHREADS, 0, s>>>(b.dcases, b.ncases, mode, trip, cap, h);
    count_launch();
}
template <typename T> void launch_stage_record(const Batch<T> &b, int si, cudaStream_t s)
{
    k_stage_record<T><<<(b.ncases + 127) / 128, 128, 0, s>>>(b.dcases, b.ncases, si);
    count_launch();
}
template <typename T> void launch_step_reset(const Batch<T> &b, cudaStream_t s)
{
    k_step_reset<T><<<(b.ncases + 127) / 128, 128, 0, s>>>(b.dcases, b.ncases);
    count_launch();
}

template void launch_loop_cond<float>(const Batch<float> &, int, int, double, cudaGraphConditionalHandle, cudaStream_t);
template void launch_stage_record<float>(const Batch<float> &, int, cudaStream_t);
template void launch_step_reset<float>(const Batch<float> &, cudaStream_t);
template void launch_loop_cond<double>(const Batch<double> &, int, int, double, cudaGraphConditionalHandle, cudaStream_t);
template void launch_stage_record<double>(const Batch<double> &, int, cudaStream_t);
template void launch_step_reset<double>(const Batch<double> &, cudaStream_t);

}  // namespace suli
