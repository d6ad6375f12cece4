// Internal helpers shared by the C-ABI translation units.
#pragma once

#include <string>

namespace fitsne {

// Records msg as the calling thread's last error and returns code.
int set_error(int code, const std::string &msg);
// 32 or 64: precision of the one-shot entry points.
int precision_bits();
// 0 when a CUDA device is usable, else records the error and returns FITSNE_E_CUDA.
int check_cuda_device();

}  // namespace fitsne
