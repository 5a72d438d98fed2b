// rz_fill_u32.cu -- fill kernels instantiated for uint32_t rasters.
#include "rz_fill.cuh"

int rz_fill_u32(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<uint32_t>(a, fn, dedup, num_sms, s);
}
