// Kernel variants with e4m3 slices (kind::f8f6f4, b <= 4; see oz_gemm.cuh).
#include "oz_gemm.cuh"

namespace ozgb {
#define OZ_DEFINE_GEMM_F8(BN, W, KC)                                                  \
    void launch_gemm_f8_##BN##_##W##_##KC(const GemmArgs &a, int g, size_t s, void *st) { \
        launch_gemm_variant<BN, W, KC, true>(a, g, s, st);                              \
    }
OZ_GEMM_F8_VARIANTS(OZ_DEFINE_GEMM_F8)
#undef OZ_DEFINE_GEMM_F8
}  // namespace ozgb
