// Kernel variants with 48-column tiles (see oz_gemm.cuh).
#include "oz_gemm.cuh"

namespace ozgb {
void launch_gemm_48_3(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<48, 3>(a, g, s, st); }
void launch_gemm_48_4(const GemmArgs &a, int g, size_t s, void *st) { launch_gemm_variant<48, 4>(a, g, s, st); }
}  // namespace ozgb
