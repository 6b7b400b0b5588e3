// engine_mixed.cu -- the mixed-precision instantiation (R = float) of the
// blob-step kernels: FP32 stress, matrix and SpMV; FP64 Jacobian inversion,
// dot-product accumulation and position accumulator.
#include "engine_impl.cuh"

namespace ffea {

template struct Launch<float>;

}  // namespace ffea
