// rz_fill_f64.cu -- fill kernels instantiated for double rasters.
#include "rz_fill.cuh"

int rz_fill_f64(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<double>(a, fn, dedup, num_sms, s);
}
