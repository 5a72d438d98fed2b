// rz_fill_f32.cu -- fill kernels instantiated for float rasters.
#include "rz_fill.cuh"

int rz_fill_f32(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<float>(a, fn, dedup, num_sms, s);
}
