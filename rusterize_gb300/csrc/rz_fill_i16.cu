// rz_fill_i16.cu -- fill and sparse-replay kernels instantiated for int16_t rasters.
#include "rz_fill.cuh"
#include "rz_replay.cuh"

int rz_fill_i16(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<int16_t>(a, fn, dedup, num_sms, s);
}

int rz_replay_i16(const rzd::ReplayArgs& a, int fn, int num_sms, cudaStream_t s) {
  return rzd::launch_replay_t<int16_t>(a, fn, num_sms, s);
}
