// Test infrastructure only (oracle): link stubs for the two CUDA entry points that
// cppSrc/neighSearch.cpp:121-141 declares.  The reference's CUDA translation unit
// (cppSrc/neighSearch_cuda.cu) does not compile against torch >= 2.x
// (`AT_DISPATCH_FLOATING_TYPES(x.type(), ...)` at cppSrc/neighSearch_cuda.cu:235,288),
// and the oracle only needs the CPU entry points `buildNeighborList`,
// `buildNeighborListUnsortedPerParticle` and `buildNeighborListAsymmetric`.
#include <torch/extension.h>
#include <utility>

std::pair<torch::Tensor, torch::Tensor> countNeighborsCUDAImpl(
    torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor,
    torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor,
    float, int32_t, int32_t, int32_t) {
  TORCH_CHECK(false, "oracle build: the reference CUDA path is not compiled");
}

std::pair<torch::Tensor, torch::Tensor> constructNeighborsCUDAImpl(
    torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor,
    torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor,
    torch::Tensor, torch::Tensor, float, int32_t, int32_t, int32_t) {
  TORCH_CHECK(false, "oracle build: the reference CUDA path is not compiled");
}
