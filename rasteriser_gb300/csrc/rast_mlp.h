// The learned many-light shader: a BF16 MLP that maps a camera-space normal and an albedo to the
// summed Lambert radiance of the context's directional lights (shading.cpp:20-34 over many
// lights), evaluated on the tensor cores (tcgen05) with FP32 accumulation. Two networks, chosen by
// RAST_OPT_MLP_NETWORK, share one layout:
//
//   input   x = [sin(f*pi*n_c), cos(f*pi*n_c) for c in xyz, f = 1..F] (6F) ++ n (3) ++ albedo (3)
//           ++ 1 ++ zeros: K features (6F + 7 in use, padded to a multiple of 16), rounded to BF16
//   hidden  h1 = relu(W1 x), h2 = relu(W2 h1): H each, rounded to BF16
//   output  o = W3 h2 (3), radiance_c = albedo_c * (o_c * out_scale)
//
//   compact (default): F = 3, K = 32, H = 32
//   wide:              F = 16, K = 112, H = 64 (the 16-frequency 64 -> 64 -> 3 network)
//
// The biases are folded into the matrices: feature 6F + 6 is the constant 1, so that column of W1
// is the first layer's bias; hidden unit H - 1 of each layer is the constant 1 (row H - 1 of W1 is
// e_(6F+6), row H - 1 of W2 is e_(H-1)), so column H - 1 of W2 and W3 holds the next layer's bias.
// The radiance is linear in the albedo for a fixed normal, so the albedo scales the output; it is
// also an input, as the model maps (normal, colour) to radiance.
//
// The compact size: trained the same way on 256-light rigs, it is about as accurate as the wide
// one (held-out mean error about 0.02/255 against 0.015/255, largest about 0.25/255 against
// 0.17/255), while every layer is two K = 16 MMAs instead of four to seven and the epilogues handle
// half the values. Hidden layers of 16 came within reach of the 0.5/255 bound the checks enforce.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#if defined(__CUDACC__)
#define RAST_HD __host__ __device__
#else
#define RAST_HD
#endif

namespace rast {

constexpr int kMlpOut = 3;        // radiance channels
constexpr int kMlpOutPad = 16;    // N of the last MMA
constexpr int kMlpRows = 128;     // fragments per tile (M of every MMA)

// Saved weights ("RMLP" blob, little endian): header, then W1 H x (6F + 7), W2 H x H, W3 3 x H as
// BF16 bit patterns (row major [out][in], biases folded in as above).
constexpr uint32_t kMlpBlobVersion = 3;  // 1: 16 frequencies, 103 inputs, one network; 2: 8, 55
struct MlpBlobHeader {
    char magic[4];          // "RMLP"
    uint32_t version;       // kMlpBlobVersion
    uint32_t n_in;          // 6F + 7
    uint32_t n_hidden;      // H
    uint32_t n_out;         // 3
    uint32_t n_freq;        // F
    uint32_t n_lights;      // lights of the rig it was trained for
    uint32_t reserved;
    uint64_t lights_hash;   // FNV-1a 64 of the rig's light records (nl * 7 floats)
    float out_scale;
    float train_loss;
};

// Byte offset of element (row, k) of a [rows][K] BF16 operand in the tensor cores' K-major,
// unswizzled shared-memory layout: 8x8 core matrices of 128 contiguous bytes (8 rows of 16 bytes),
// row groups 128 bytes apart, K groups rows*16 bytes apart. The matrix descriptor then carries
// leading (K-direction) byte offset rows*16 and stride (row-direction) byte offset 128.
RAST_HD constexpr uint32_t core_offset(uint32_t rows, uint32_t row, uint32_t k) {
    return (k >> 3) * rows * 16u + (row >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// One network's sizes. Parameters (row major [out][in]) in one array: W1 H x K, W2 H x H, W3 3 x H.
// Fixed entries: W1 columns >= 6F + 7 (0), W1 row H - 1 (e_(6F+6)) and W2 row H - 1 (e_(H-1)).
// The device image holds W1, W2 and W3 as B operands in the core layout (W3 padded to 16 rows),
// then the output scale in a 16-byte word; the checks' light table (MlpCheckTable) follows it.
template <int F_, int H_>
struct MlpNet {
    static constexpr int kFreq = F_;               // Fourier frequencies per normal component
    static constexpr int kFeat = 6 * F_ + 7;       // features in use, the constant included
    static constexpr int kConst = 6 * F_ + 6;      // the constant-1 feature
    static constexpr int kIn = (kFeat + 15) / 16 * 16;  // padded input features (K of layer 1)
    static constexpr int kHid = H_;                // hidden width
    static constexpr int kUnit1 = H_ - 1;          // the constant-1 hidden unit of both hidden layers
    static constexpr int kPW1 = 0;
    static constexpr int kPW2 = kPW1 + kHid * kIn;
    static constexpr int kPW3 = kPW2 + kHid * kHid;
    static constexpr int kParams = kPW3 + kMlpOut * kHid;
    static constexpr uint32_t kW1Off = 0;
    static constexpr uint32_t kW2Off = kW1Off + 2u * kHid * kIn;
    static constexpr uint32_t kW3Off = kW2Off + 2u * kHid * kHid;
    static constexpr uint32_t kScaleOff = kW3Off + 2u * kMlpOutPad * kHid;
    static constexpr uint32_t kImageBytes = kScaleOff + 16u;
    static constexpr size_t kBlobBytes =
        sizeof(MlpBlobHeader) + sizeof(uint16_t) * (kHid * kFeat + kHid * kHid + kMlpOut * kHid);
    RAST_HD static constexpr bool fixed(int p) {
        return p < kPW2 ? ((p % kIn) >= kFeat || p / kIn == kUnit1) : (p < kPW3 && (p - kPW2) / kHid == kUnit1);
    }
    static_assert(kIn % 16 == 0 && kHid % 16 == 0 && kW2Off % 16 == 0 && kW3Off % 16 == 0 && kScaleOff % 16 == 0,
                  "whole K steps and 16-byte aligned operands");
};
using MlpCompact = MlpNet<3, 32>;
using MlpWide = MlpNet<16, 64>;
constexpr int kMlpNetCompact = 0, kMlpNetWide = 1;  // RAST_OPT_MLP_NETWORK values

// Runs f(N{}) with the network type of `net` (kMlpNetCompact or kMlpNetWide).
template <class Fn>
inline auto with_mlp_net(int net, Fn&& f) {
    return net == kMlpNetWide ? f(MlpWide{}) : f(MlpCompact{});
}

// The light table of the learned shader's checks, built with the image for the rig the weights
// belong to and stored right after it on the device: dirI[l] = (-dir xyz, I r), gb[l] = (I g, I b)
// for the first kMlpCheckLights lights (a rig with more lights is read from the light records).
constexpr int kMlpCheckLights = 512;
struct MlpCheckTable {
    float dirI[kMlpCheckLights][4];
    float gb[kMlpCheckLights][2];
};
static_assert(sizeof(MlpCheckTable) % 16 == 0, "16-byte units");

// FNV-1a 64 of n light records (7 floats each), identifying the rig a model was trained for.
inline uint64_t lights_hash(const float* lights7, int32_t n) {
    uint64_t h = 0xcbf29ce484222325ull;
    const unsigned char* b = reinterpret_cast<const unsigned char*>(lights7);
    for (size_t i = 0; i < sizeof(float) * 7 * (size_t)(n > 0 ? n : 0); ++i) {
        h ^= b[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

// Launchers (rast_shade.cu). Each returns its number of kernel launches, or -1.
int launch_mlp_samples(float* out, int64_t n, uint64_t seed, const float* lights, int nl, cudaStream_t stream);
int launch_mlp_train_step(int net, const float* q, const float* samples, int64_t n, int64_t first, int n_cta,
                          float out_scale, float grad_scale, float* grad, float* loss, cudaStream_t stream);
int launch_mlp_adam(int net, float* w, float* q, float* m, float* v, const float* grad, int n_part, float lr,
                    float beta1, float beta2, float eps, float c1, float c2, const float* loss_part, float* loss_out,
                    cudaStream_t stream);
// Shades n records (normal xyz, albedo rgb at src + i*stride) into out (n * 3 radiance floats)
// with the learned (exact = false; network `net`, image `mlp`) or the exact shader. gbuf / count /
// index: scratch for ceil(n/1024) blocks of records.
int launch_mlp_eval(int net, const float* src, int stride, int64_t n, bool exact, float4* gbuf, uint32_t* count,
                    uint32_t* index, const float* lights, int nl, const void* mlp, uint32_t* counters, int n_sm,
                    float* out, cudaStream_t stream);
int train_batch_per_cta();

}  // namespace rast
