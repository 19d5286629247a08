// TEST INFRASTRUCTURE ONLY. The reference was written against a Thrust that still shipped
// thrust::optional (its deps/thrust submodule, version unpinned); the CCCL 3 Thrust of CUDA 13
// dropped that header. The reference uses only construction, emplace, operator bool, -> and
// nullopt, which std::optional provides with the same meaning.
#pragma once
#include <optional>
namespace thrust {
using std::nullopt;
using std::optional;
}  // namespace thrust
