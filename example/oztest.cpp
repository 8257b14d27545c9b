// Minimal consumer of the drop-in API: the same calls an Oz-AIE user makes.
// Prints max |C - exact| for an all-ones 256 x 512 x 128 product (exact value K).
#include <cmath>
#include <cstdio>
#include <vector>

#include "oz_aie.h"

int main() {
    const int M = 256, N = 512, K = 128;
    const int setup_status = oz_aie::ozAIE_setup(M, N, K, oz_aie::Mode::accurate);
    if (setup_status > 0) {
        std::fprintf(stderr, "setup failed: %d\n", setup_status);
        return setup_status;
    }
    std::vector<double> A(static_cast<size_t>(M) * K, 1.0), B(static_cast<size_t>(K) * N, 1.0),
        C(static_cast<size_t>(M) * N, 0.0);
    const int rc = oz_aie::ozAIE_DGEMM(M, N, K, A.data(), B.data(), C.data());
    if (rc != 0) {
        std::fprintf(stderr, "DGEMM failed: %d\n", rc);
        return rc;
    }
    double err = 0.0;
    for (double c : C) err = std::fmax(err, std::fabs(c - K));
    std::printf("max |C - %d| = %g\n", K, err);
    return err == 0.0 ? 0 : 1;
}
