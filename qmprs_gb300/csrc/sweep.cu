// (d) end of a sweep, for every state at once: the fidelity after the
// sweep, |<target|C|0>| / ||target||, is the nuclear norm of the last
// step's environment (the trace Re Tr(W^H E) of its new gate) over the
// target norm (reference qmprs/synthesis/mps_encoding/sequential.py:509-541
// reports the same overlap after each sweep).  States that reach the stop
// fidelity leave the active set.
#include "device_common.cuh"

// After a sweep: record |<target|C|0>| / ||target|| and retire finished states.
__global__ void k_sweep_finish(int B, int sweep, int num_sweeps, const double* nuc, const double2* tnorm2,
                               double* sweep_fid, int* sweeps_done, int* active, double stop_fid,
                               int* num_active) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    if (!active[b]) continue;
    const double f = nuc[b] / sqrt(tnorm2[b].x);
    sweep_fid[(int64_t)b * num_sweeps + sweep] = f;
    sweeps_done[b] = sweep + 1;
    if (stop_fid > 0.0 && f >= stop_fid) active[b] = 0;
    else atomicAdd(num_active, 1);
  }
}

void launch_sweep_finish(int B, int sweep, int num_sweeps, const double* nuc, const double2* tnorm2,
                         double* sweep_fid, int* sweeps_done, int* active, double stop_fid,
                         int* num_active, cudaStream_t s) {
  qm_note_launch();
  k_sweep_finish<<<(B + 127) / 128, 128, 0, s>>>(B, sweep, num_sweeps, nuc, tnorm2, sweep_fid,
                                                 sweeps_done, active, stop_fid, num_active);
}
