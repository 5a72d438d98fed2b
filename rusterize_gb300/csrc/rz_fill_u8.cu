// rz_fill_u8.cu -- fill kernels instantiated for uint8_t rasters.
#include "rz_fill.cuh"

int rz_fill_u8(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<uint8_t>(a, fn, dedup, num_sms, s);
}
