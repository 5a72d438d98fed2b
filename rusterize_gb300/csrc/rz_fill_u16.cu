// rz_fill_u16.cu -- fill kernels instantiated for uint16_t rasters.
#include "rz_fill.cuh"

int rz_fill_u16(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<uint16_t>(a, fn, dedup, num_sms, s);
}
