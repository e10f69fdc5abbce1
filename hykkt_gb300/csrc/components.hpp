// Component entry points (device) used by the C ABI.
#pragma once

#include <cuda_runtime.h>

namespace hykkt {

void map_index(int n, const int* d_map, const double* d_old, double* d_new, cudaStream_t st);
void ruiz_scale(int its, int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v, const int* bt_i,
                const int* bt_j, double* b_v, const int* b_i, const int* b_j, double* rhs1, double* rhs2,
                double* max_d, cudaStream_t st);

// Same sweeps with the scale vector in a fixed device array (no allocation);
// n + m <= ruiz_noalloc_max_rows().
void ruiz_scale_noalloc(int its, int n, int m, double* a_v, const int* a_i, const int* a_j, double* bt_v,
                        const int* bt_i, const int* bt_j, double* b_v, const int* b_i, const int* b_j, double* rhs1,
                        double* rhs2, double* max_d, cudaStream_t st);
int ruiz_noalloc_max_rows();

double fp64_peak_tflops();
// mode 0: DFMA chains (fp64_peak_tflops); 1: FP64 mma.sync m8n8k4; 2: both kinds in one kernel
double fp64_probe_tflops(int mode);

}  // namespace hykkt
