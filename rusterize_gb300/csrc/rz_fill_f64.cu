// rz_fill_f64.cu -- fill and sparse-replay kernels instantiated for double rasters.
#include "rz_fill.cuh"
#include "rz_replay.cuh"

int rz_fill_f64(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<double>(a, fn, dedup, num_sms, s);
}

int rz_replay_f64(const rzd::ReplayArgs& a, int fn, int num_sms, cudaStream_t s) {
  return rzd::launch_replay_t<double>(a, fn, num_sms, s);
}
