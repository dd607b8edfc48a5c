// A small multilayer perceptron on the GPU (device/mlp.cu): the warm-start surrogate that maps
// model descriptors to a steady temperature map.  Parameters and activations are BF16,
// products accumulate in FP32, Adam keeps FP32 master weights.  No CUDA types appear here.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

namespace psim::gpu {

class Mlp {
public:
    // widths[0] inputs, widths[1..n-1] hidden (GELU), widths[n] outputs (linear).  Weights are
    // drawn N(0, 1/fan_in) from `seed`, biases are zero.
    Mlp(const std::vector<int>& widths, std::uint64_t seed);
    ~Mlp();
    Mlp(const Mlp&) = delete;
    Mlp& operator=(const Mlp&) = delete;

    const std::vector<int>& widths() const noexcept { return widths_; }
    std::size_t n_params() const noexcept { return n_params_; }
    // FP32 master parameters, per layer W [in][out] then b [out]; set also refreshes the BF16 copy.
    void get_params(float* out) const;
    void set_params(const float* in);
    // Mean squared error over x [n][in] -> y [n][out] and its gradient for every parameter.
    float gradients(const float* x, const float* y, int n, float* grads);
    // Adam steps (beta 0.9 / 0.999, eps 1e-8) over shuffled mini-batches; returns the last
    // epoch's mean loss.
    float train(const float* x, const float* y, int n, int batch, int epochs, float lr, std::uint64_t seed);
    void predict(const float* x, int n, float* y);

    struct Impl;// device buffers (device/mlp.cu)

private:
    std::vector<int> widths_;
    std::size_t n_params_{ 0 };
    std::unique_ptr<Impl> impl_;
};

}// namespace psim::gpu
