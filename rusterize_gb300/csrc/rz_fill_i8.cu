// rz_fill_i8.cu -- fill kernels instantiated for int8_t rasters.
#include "rz_fill.cuh"

int rz_fill_i8(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<int8_t>(a, fn, dedup, num_sms, s);
}
