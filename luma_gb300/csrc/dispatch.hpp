// Runtime lattice/precision dispatch to the templated launchers.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "device.cuh"

namespace luma {

template <class F>
cudaError_t dispatch(int Q, int prec, F &&f) {
    if (prec == LUMA_PREC_FP64) {
        if (Q == 9) return f(std::integral_constant<int, 9>{}, P64{});
        if (Q == 19) return f(std::integral_constant<int, 19>{}, P64{});
        return f(std::integral_constant<int, 27>{}, P64{});
    }
    if (Q == 9) return f(std::integral_constant<int, 9>{}, P32{});
    if (Q == 19) return f(std::integral_constant<int, 19>{}, P32{});
    return f(std::integral_constant<int, 27>{}, P32{});
}

}  // namespace luma
