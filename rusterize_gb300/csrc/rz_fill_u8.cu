// rz_fill_u8.cu -- fill and sparse-replay kernels instantiated for uint8_t rasters.
#include "rz_fill.cuh"
#include "rz_replay.cuh"

int rz_fill_u8(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<uint8_t>(a, fn, dedup, num_sms, s);
}

int rz_replay_u8(const rzd::ReplayArgs& a, int fn, int num_sms, cudaStream_t s) {
  return rzd::launch_replay_t<uint8_t>(a, fn, num_sms, s);
}
