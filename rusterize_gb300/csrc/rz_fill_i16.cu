// rz_fill_i16.cu -- fill kernels instantiated for int16_t rasters.
#include "rz_fill.cuh"

int rz_fill_i16(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<int16_t>(a, fn, dedup, num_sms, s);
}
