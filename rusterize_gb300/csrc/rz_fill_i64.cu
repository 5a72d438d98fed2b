// rz_fill_i64.cu -- fill kernels instantiated for int64_t rasters.
#include "rz_fill.cuh"

int rz_fill_i64(const rzd::FillArgs& a, int fn, bool dedup, int num_sms, cudaStream_t s) {
  return rzd::launch_fill_t<int64_t>(a, fn, dedup, num_sms, s);
}
