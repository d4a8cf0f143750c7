// sincos_reduced.cuh - sin and cos of a phase for the far-field pattern kernels.
#pragma once

namespace emlab {

// sin and cos of psi: Cody-Waite reduction by 2 pi (2 pi split into its nearest float and the
// remainder), then the hardware approximations on [-pi, pi]. Absolute error about |psi| 2^-24 +
// 2^-21 (6e-6 at |psi| = 100), for pattern evaluations that do not restate a reference shader.
__device__ __forceinline__ void sincos_reduced(float psi, float* s, float* c) {
    const float n = rintf(psi * 0.159154943091895336f);
    float r = fmaf(-n, 6.28318548202514648f, psi);
    r = fmaf(-n, -1.74845560007441e-07f, r);
    __sincosf(r, s, c);
}

}  // namespace emlab
