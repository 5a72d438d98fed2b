// rz_fill_f32.cu -- fill and sparse-replay kernels instantiated for float rasters.
#include "rz_fill.cuh"
#include "rz_replay.cuh"

int rz_fill_f32(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<float>(a, fn, dedup, num_sms, s);
}

int rz_replay_f32(const rzd::ReplayArgs& a, int fn, int num_sms, cudaStream_t s) {
  return rzd::launch_replay_t<float>(a, fn, num_sms, s);
}
