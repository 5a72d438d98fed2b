// rz_fill_i32.cu -- fill and sparse-replay kernels instantiated for int32_t rasters.
#include "rz_fill.cuh"
#include "rz_replay.cuh"

int rz_fill_i32(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<int32_t>(a, fn, dedup, num_sms, s);
}

int rz_replay_i32(const rzd::ReplayArgs& a, int fn, int num_sms, cudaStream_t s) {
  return rzd::launch_replay_t<int32_t>(a, fn, num_sms, s);
}
