// idg_host.h -- host-side helpers shared by the C ABI translation units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/idg_gb300.h"

namespace idg {

// Records the calling thread's error text and returns `code`.
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define IDG_CUDA(call)                                                                                                 \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return ::idg::cuda_fail(e_, #call);                                                     \
    } while (0)

// Per-device words: the device check word (kernels OR bits into it) and the
// persistent kernels' work counter.
struct DeviceWords {
    unsigned *status = nullptr;
    int *counter = nullptr;
};
int device_words(DeviceWords *out);

int check_params(const idg_params *p, bool need_fft_size = false);

} // namespace idg
