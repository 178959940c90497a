// The learned many-light shader: a BF16 MLP that maps a camera-space normal and an albedo to the
// summed Lambert radiance of the context's directional lights (shading.cpp:20-34 over many
// lights), evaluated on the tensor cores (tcgen05) with FP32 accumulation.
//
//   input   x = [sin(f*pi*n_c), cos(f*pi*n_c) for c in xyz, f = 1..3] (18) ++ n (3) ++ albedo (3)
//           ++ 1 ++ zeros (7): 32 features, rounded to BF16
//   hidden  h1 = relu(W1 x), h2 = relu(W2 h1): 32 each, rounded to BF16
//   output  o = W3 h2 (3), radiance_c = albedo_c * (o_c * out_scale)
//
// The biases are folded into the matrices: feature 24 is the constant 1, so column 24 of W1 is
// the first layer's bias; hidden unit 31 of each layer is the constant 1 (row 31 of W1 is e_24,
// row 31 of W2 is e_31), so column 31 of W2 and W3 holds the next layer's bias. The radiance is
// linear in the albedo for a fixed normal, so the albedo scales the output; it is also an input,
// as the model maps (normal, colour) to radiance.
//
// The size: trained the same way on 256-light rigs, this network is as accurate as one with 8
// frequencies and two hidden layers of 64 (held-out mean error about 0.02/255, largest about
// 0.25/255), while every layer is two K = 16 MMAs instead of four and the epilogues handle half
// the values. Hidden layers of 16 came within reach of the 0.5/255 bound the checks enforce.
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

constexpr int kMlpIn = 32;        // padded input features (K of layer 1)
constexpr int kMlpFeat = 25;      // features in use, the constant included
constexpr int kMlpConst = 24;     // the constant-1 feature
constexpr int kMlpFreq = 3;       // Fourier frequencies per normal component
constexpr int kMlpHid = 32;       // hidden width
constexpr int kMlpUnit1 = kMlpHid - 1;  // the constant-1 hidden unit of both hidden layers
constexpr int kMlpOut = 3;        // radiance channels
constexpr int kMlpOutPad = 16;    // N of the last MMA
constexpr int kMlpRows = 128;     // fragments per tile (M of every MMA)

// Parameters (row major [out][in]) in one array: W1 32x32, W2 32x32, W3 3x32. Fixed entries:
// W1 columns >= 25 (0), W1 row 31 (e_24) and W2 row 31 (e_31).
constexpr int kPW1 = 0;
constexpr int kPW2 = kPW1 + kMlpHid * kMlpIn;
constexpr int kPW3 = kPW2 + kMlpHid * kMlpHid;
constexpr int kMlpParams = kPW3 + kMlpOut * kMlpHid;

RAST_HD constexpr bool mlp_param_fixed(int p) {
    return p < kPW2 ? ((p % kMlpIn) >= kMlpFeat || p / kMlpIn == kMlpUnit1)
                    : (p < kPW3 && (p - kPW2) / kMlpHid == kMlpUnit1);
}

// Byte offset of element (row, k) of a [rows][K] BF16 operand in the tensor cores' K-major,
// unswizzled shared-memory layout: 8x8 core matrices of 128 contiguous bytes (8 rows of 16 bytes),
// row groups 128 bytes apart, K groups rows*16 bytes apart. The matrix descriptor then carries
// leading (K-direction) byte offset rows*16 and stride (row-direction) byte offset 128.
RAST_HD constexpr uint32_t core_offset(uint32_t rows, uint32_t row, uint32_t k) {
    return (k >> 3) * rows * 16u + (row >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// The weights as the shading kernel copies them into shared memory, and the output scale. Built
// from the parameters by the training pass or from a saved blob.
struct MlpImage {
    uint16_t w1[kMlpHid * kMlpIn];      // layer 1 B operand, 32 rows x K 32, core layout
    uint16_t w2[kMlpHid * kMlpHid];     // layer 2 B operand, 32 x 32
    uint16_t w3[kMlpOutPad * kMlpHid];  // layer 3 B operand, 16 x 32 (rows 3.. zero)
    float out_scale;
    float reserved[3];
};
static_assert(sizeof(MlpImage) % 16 == 0, "MlpImage is copied in 16-byte units");

// The light table of the learned shader's checks, built with the image for the rig the weights
// belong to and stored right after it on the device: dirI[l] = (-dir xyz, I r), gb[l] = (I g, I b)
// for the first kMlpCheckLights lights (a rig with more lights is read from the light records).
constexpr int kMlpCheckLights = 512;
struct MlpCheckTable {
    float dirI[kMlpCheckLights][4];
    float gb[kMlpCheckLights][2];
};
static_assert(sizeof(MlpImage) % 16 == 0 && sizeof(MlpCheckTable) % 16 == 0, "16-byte units");
constexpr uint32_t kMlpWeightBytes = sizeof(uint16_t) * (kMlpHid * kMlpIn + kMlpHid * kMlpHid + kMlpOutPad * kMlpHid);

// Saved weights ("RMLP" blob, little endian): header, then W1 32x25, W2 32x32, W3 3x32 as BF16
// bit patterns (row major [out][in], biases folded in as above).
constexpr uint32_t kMlpBlobVersion = 3;  // 1: 16 frequencies, 103 inputs; 2: 8, 55 inputs, 64 hidden
struct MlpBlobHeader {
    char magic[4];          // "RMLP"
    uint32_t version;       // kMlpBlobVersion
    uint32_t n_in;          // 25
    uint32_t n_hidden;      // 32
    uint32_t n_out;         // 3
    uint32_t n_freq;        // 3
    uint32_t n_lights;      // lights of the rig it was trained for
    uint32_t reserved;
    uint64_t lights_hash;   // FNV-1a 64 of the rig's light records (nl * 7 floats)
    float out_scale;
    float train_loss;
};
constexpr size_t kMlpBlobBytes = sizeof(MlpBlobHeader) +
                                 sizeof(uint16_t) * (kMlpHid * kMlpFeat + kMlpHid * kMlpHid + kMlpOut * kMlpHid);

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
int launch_mlp_train_step(const float* q, const float* samples, int64_t n, int64_t first, int n_cta, float out_scale,
                          float grad_scale, float* grad, float* loss, cudaStream_t stream);
int launch_mlp_adam(float* w, float* q, float* m, float* v, const float* grad, int n_part, float lr, float beta1,
                    float beta2, float eps, float c1, float c2, const float* loss_part, float* loss_out,
                    cudaStream_t stream);
// Shades n records (normal xyz, albedo rgb at src + i*stride) into out (n * 3 radiance floats)
// with the learned (exact = false) or the exact shader. gbuf / count / index: scratch for
// ceil(n/1024) blocks of records.
int launch_mlp_eval(const float* src, int stride, int64_t n, bool exact, float4* gbuf, uint32_t* count,
                    uint32_t* index, const float* lights, int nl, const void* mlp, uint32_t* counters, int n_sm,
                    float* out, cudaStream_t stream);
int train_batch_per_cta();

}  // namespace rast
