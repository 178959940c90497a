// Host side of the learned many-light shader: training orchestration, the weight image the
// tensor-core kernel copies into shared memory, the "RMLP" blob, and evaluation entry points.
// The kernels are in rast_shade.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "rast_context.h"

using namespace rast;

namespace {

// A device buffer freed when it goes out of scope (the training and evaluation temporaries).
struct TempBuf : DevBuf {
    TempBuf() = default;
    TempBuf(const TempBuf&) = delete;
    TempBuf& operator=(const TempBuf&) = delete;
    ~TempBuf() { release(); }
};

// BF16 bit pattern of f, rounded to nearest even (NaN to a quiet NaN).
uint16_t bf16_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, sizeof u);
    if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x7FFFFFu)) return 0x7FC0;
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

float bf16_value(uint16_t b) {
    const uint32_t u = (uint32_t)b << 16;
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
}

float round_bf16(float f) { return bf16_value(bf16_bits(f)); }

// The device image of network N (its layout in MlpNet) from the rounded parameters.
template <class N>
std::vector<unsigned char> pack_image(const std::vector<float>& q, float scale) {
    std::vector<unsigned char> im(N::kImageBytes, 0);
    auto put = [&](uint32_t off, uint32_t rows, int n, int k, float v) {
        const uint16_t b = bf16_bits(v);
        std::memcpy(im.data() + off + core_offset(rows, (uint32_t)n, (uint32_t)k), &b, 2);
    };
    for (int n = 0; n < N::kHid; ++n)
        for (int k = 0; k < N::kIn; ++k) put(N::kW1Off, N::kHid, n, k, q[N::kPW1 + n * N::kIn + k]);
    for (int n = 0; n < N::kHid; ++n)
        for (int k = 0; k < N::kHid; ++k) put(N::kW2Off, N::kHid, n, k, q[N::kPW2 + n * N::kHid + k]);
    for (int n = 0; n < kMlpOut; ++n)
        for (int k = 0; k < N::kHid; ++k) put(N::kW3Off, kMlpOutPad, n, k, q[N::kPW3 + n * N::kHid + k]);
    std::memcpy(im.data() + N::kScaleOff, &scale, sizeof scale);
    return im;
}

// Upper bound of the radiance per unit albedo: the largest channel of sum(I * colour) / pi.
float output_scale(const std::vector<float>& lights, int nl) {
    double s[3] = {0, 0, 0};
    for (int l = 0; l < nl; ++l)
        for (int c = 0; c < 3; ++c) s[c] += (double)lights[7 * l + 3] * lights[7 * l + 4 + c];
    const double m = std::max(s[0], std::max(s[1], s[2])) / 3.14159265358979323846;
    return m > 0 ? (float)m : 1.f;
}

uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// He-uniform weights; zero biases (W1 column kConst, W2 and W3 column kUnit1); the constant units
// (W1 row kUnit1 = e_kConst, W2 row kUnit1 = e_kUnit1) and zero padding columns.
template <class N>
std::vector<float> init_params(uint64_t seed) {
    std::vector<float> w(N::kParams, 0.f);
    uint64_t st = seed * 0x2545F4914F6CDD1Dull + 7;
    auto uni = [&](float a) { return a * (2.f * (float)((splitmix(st) >> 40) * 0x1p-24) - 1.f); };
    const float a1 = std::sqrt(6.f / N::kConst), a2 = std::sqrt(6.f / N::kHid), a3 = 0.5f * std::sqrt(6.f / N::kHid);
    for (int n = 0; n < N::kUnit1; ++n)
        for (int k = 0; k < N::kConst; ++k) w[N::kPW1 + n * N::kIn + k] = uni(a1);
    w[N::kPW1 + N::kUnit1 * N::kIn + N::kConst] = 1.f;
    for (int n = 0; n < N::kUnit1; ++n)
        for (int k = 0; k < N::kUnit1; ++k) w[N::kPW2 + n * N::kHid + k] = uni(a2);
    w[N::kPW2 + N::kUnit1 * N::kHid + N::kUnit1] = 1.f;
    for (int n = 0; n < kMlpOut; ++n)
        for (int k = 0; k < N::kUnit1; ++k) w[N::kPW3 + n * N::kHid + k] = uni(a3);
    return w;
}

std::vector<float> rounded(const std::vector<float>& w) {
    std::vector<float> q(w.size());
    for (size_t p = 0; p < w.size(); ++p) q[p] = round_bf16(w[p]);
    return q;
}

// The checks' light table for the rig (the first kMlpCheckLights lights).
void pack_check_table(const std::vector<float>& lights, int nl, MlpCheckTable& t) {
    std::memset(&t, 0, sizeof t);
    for (int l = 0; l < nl && l < kMlpCheckLights; ++l) {
        const float* P = lights.data() + 7 * (size_t)l;
        const float I = P[3];
        t.dirI[l][0] = -P[0];
        t.dirI[l][1] = -P[1];
        t.dirI[l][2] = -P[2];
        t.dirI[l][3] = I * P[4];
        t.gb[l][0] = I * P[5];
        t.gb[l][1] = I * P[6];
    }
}

template <class N>
rast_status install(rast_ctx* c, const std::vector<float>& q, float scale, float loss) {
    const std::vector<unsigned char> im = pack_image<N>(q, scale);
    MlpCheckTable tab;
    pack_check_table(c->lights_host, c->nl, tab);
    RAST_CUDA(c, c->mlp_image.reserve(N::kImageBytes + sizeof(MlpCheckTable)));
    RAST_CUDA(c, cudaMemcpy(c->mlp_image.ptr, im.data(), im.size(), cudaMemcpyHostToDevice));
    RAST_CUDA(c, cudaMemcpy(static_cast<char*>(c->mlp_image.ptr) + N::kImageBytes, &tab, sizeof tab,
                            cudaMemcpyHostToDevice));
    c->mlp_net = std::is_same<N, MlpWide>::value ? kMlpNetWide : kMlpNetCompact;
    c->mlp_q = q;
    c->mlp_scale = scale;
    c->mlp_loss = loss;
    c->mlp_nl = c->nl;
    c->mlp_lights_hash = lights_hash(c->lights_host.data(), c->nl);
    c->mlp_ready = true;
    return RAST_OK;
}

// Evaluation through the shading kernels on device-resident records (stride floats apart).
rast_status eval_device(rast_ctx* c, const float* d_src, int stride, int64_t n, bool exact, float* d_out) {
    const int64_t blocks = (n + kShadeBlock - 1) / kShadeBlock;
    TempBuf gbuf, count, index, counters;
    RAST_CUDA(c, gbuf.reserve(2 * sizeof(float4) * (size_t)blocks * kShadeBlock));
    RAST_CUDA(c, count.reserve(sizeof(uint32_t) * (size_t)blocks));
    RAST_CUDA(c, index.reserve(sizeof(uint32_t) * (size_t)kShadeIndexWords(blocks)));
    RAST_CUDA(c, counters.reserve(sizeof(uint32_t) * kCounterHeader));
    RAST_CUDA(c, cudaMemsetAsync(counters.ptr, 0, sizeof(uint32_t) * kCounterHeader, c->stream));
    if (launch_mlp_eval(c->mlp_net, d_src, stride, n, exact, gbuf.as<float4>(), count.as<uint32_t>(), index.as<uint32_t>(),
                        c->lights.as<float>(), c->nl, c->mlp_image.ptr, counters.as<uint32_t>(), c->n_sm, d_out,
                        c->stream) < 0)
        return cuda_fail(c, cudaGetLastError(), "MLP evaluation launch");
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    uint32_t status = 0;
    RAST_CUDA(c, cudaMemcpy(&status, counters.as<uint32_t>() + 1, sizeof status, cudaMemcpyDeviceToHost));
    if (status & STATUS_SHADE_TIMEOUT)
        return fail(c, RAST_ERR_INTERNAL, "learned shader: a tensor-core MMA did not complete in time");
    if (status) return fail(c, RAST_ERR_INTERNAL, "MLP evaluation: device status " + std::to_string(status));
    return RAST_OK;
}

// Trains network N on the context's rig (settings checked by the caller) and installs it.
template <class N>
rast_status train(rast_ctx* c, const rast_mlp_train_desc& d, float out[4]) {
    const int net = std::is_same<N, MlpWide>::value ? kMlpNetWide : kMlpNetCompact;
    const auto t0 = std::chrono::steady_clock::now();

    const int64_t n = d.samples, nh = d.holdout, B = (int64_t)train_batch_per_cta() * d.ctas;
    const int64_t per_epoch = (n + B - 1) / B, steps = per_epoch * d.epochs;
    TempBuf samples, w, q, m, v, grad, loss_part, loss_steps, hout;
    RAST_CUDA(c, samples.reserve(sizeof(float) * 9 * (size_t)(n + nh)));
    for (DevBuf* b : {&w, &q, &m, &v}) RAST_CUDA(c, b->reserve(sizeof(float) * N::kParams));
    RAST_CUDA(c, grad.reserve(sizeof(float) * N::kParams * (size_t)d.ctas));
    RAST_CUDA(c, loss_part.reserve(sizeof(float) * (size_t)d.ctas));
    RAST_CUDA(c, loss_steps.reserve(sizeof(float) * (size_t)steps));

    const std::vector<float> w0 = init_params<N>(d.seed), q0 = rounded(w0);
    RAST_CUDA(c, cudaMemcpy(w.ptr, w0.data(), sizeof(float) * N::kParams, cudaMemcpyHostToDevice));
    RAST_CUDA(c, cudaMemcpy(q.ptr, q0.data(), sizeof(float) * N::kParams, cudaMemcpyHostToDevice));
    RAST_CUDA(c, cudaMemset(m.ptr, 0, sizeof(float) * N::kParams));
    RAST_CUDA(c, cudaMemset(v.ptr, 0, sizeof(float) * N::kParams));
    if (launch_mlp_samples(samples.as<float>(), n + nh, d.seed, c->lights.as<float>(), c->nl, c->stream) < 0)
        return cuda_fail(c, cudaGetLastError(), "training samples");

    const float scale = output_scale(c->lights_host, c->nl);
    const float grad_scale = 2.f / (3.f * (float)B * scale * scale);
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    double b1t = 1.0, b2t = 1.0;
    for (int64_t step = 0; step < steps; ++step) {
        const int64_t first = (step * B) % n;
        if (launch_mlp_train_step(net, q.as<float>(), samples.as<float>(), n, first, d.ctas, scale, grad_scale,
                                  grad.as<float>(), loss_part.as<float>(), c->stream) < 0)
            return cuda_fail(c, cudaGetLastError(), "training step");
        b1t *= beta1;
        b2t *= beta2;
        const double frac = steps > 1 ? (double)step / (double)(steps - 1) : 1.0;
        const float lr = d.lr * (float)(0.01 + 0.99 * 0.5 * (1.0 + std::cos(3.14159265358979323846 * frac)));
        if (launch_mlp_adam(net, w.as<float>(), q.as<float>(), m.as<float>(), v.as<float>(), grad.as<float>(), d.ctas, lr,
                            beta1, beta2, eps, (float)(1.0 - b1t), (float)(1.0 - b2t), loss_part.as<float>(),
                            loss_steps.as<float>() + step, c->stream) < 0)
            return cuda_fail(c, cudaGetLastError(), "optimiser step");
    }
    std::vector<float> qh(N::kParams), losses((size_t)steps);
    RAST_CUDA(c, cudaMemcpyAsync(qh.data(), q.ptr, sizeof(float) * N::kParams, cudaMemcpyDeviceToHost, c->stream));
    RAST_CUDA(c, cudaMemcpyAsync(losses.data(), loss_steps.ptr, sizeof(float) * steps, cudaMemcpyDeviceToHost,
                                 c->stream));
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    double last = 0;
    for (int64_t s = steps - per_epoch; s < steps; ++s) last += losses[(size_t)s];
    const float mse = (float)(last / ((double)per_epoch * 3.0 * (double)B));
    rast_status st = install<N>(c, qh, scale, mse);
    if (st != RAST_OK) return st;

    float mean_err = 0.f, max_err = 0.f;
    if (nh > 0) {
        RAST_CUDA(c, hout.reserve(sizeof(float) * 3 * (size_t)nh));
        st = eval_device(c, samples.as<float>() + 9 * n, 9, nh, false, hout.as<float>());
        if (st != RAST_OK) return st;
        std::vector<float> pred(3 * (size_t)nh), ref(9 * (size_t)nh);
        RAST_CUDA(c, cudaMemcpy(pred.data(), hout.ptr, sizeof(float) * pred.size(), cudaMemcpyDeviceToHost));
        RAST_CUDA(c, cudaMemcpy(ref.data(), samples.as<float>() + 9 * n, sizeof(float) * ref.size(),
                                cudaMemcpyDeviceToHost));
        double sum = 0;
        for (int64_t i = 0; i < nh; ++i)
            for (int ch = 0; ch < 3; ++ch) {
                const float e = std::fabs(pred[3 * i + ch] - ref[9 * i + 6 + ch]);
                sum += e;
                max_err = std::max(max_err, e);
            }
        mean_err = (float)(sum / (3.0 * (double)nh));
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (out) {
        out[0] = mse;
        out[1] = mean_err;
        out[2] = max_err;
        out[3] = (float)secs;
    }
    return RAST_OK;
}

}  // namespace

extern "C" {

rast_status rast_mlp_train(rast_ctx* c, const rast_mlp_train_desc* desc, float out[4]) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (out)
        for (int i = 0; i < 4; ++i) out[i] = 0.f;
    if (c->nl < 1) return fail(c, RAST_ERR_INVALID_ARG, "set the lights before training");
    rast_mlp_train_desc d = {};
    if (desc) d = *desc;
    if (d.samples == 0) d.samples = 4194304;
    if (d.holdout == 0) d.holdout = 65536;
    if (d.epochs == 0) d.epochs = 24;
    if (d.ctas == 0) d.ctas = c->n_sm;
    if (d.lr == 0.f) d.lr = 3e-3f;
    if (d.seed == 0) d.seed = 1;
    if (d.samples < 1024 || d.samples > ((int64_t)1 << 28) || d.holdout < 0 || d.holdout > ((int64_t)1 << 24) ||
        d.epochs < 1 || d.epochs > 10000 || d.ctas < 1 || d.ctas > 4096 || !(d.lr > 0.f && d.lr <= 1.f))
        return fail(c, RAST_ERR_INVALID_ARG, "training settings out of range");
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    return with_mlp_net(c->mlp_train_net, [&](auto n) { return train<decltype(n)>(c, d, out); });
}

rast_status rast_mlp_save(rast_ctx* c, void* buf, size_t cap, size_t* size) {
    if (!c || !size) return RAST_ERR_INVALID_ARG;
    const int net = c->mlp_ready ? c->mlp_net : c->mlp_train_net;
    *size = with_mlp_net(net, [](auto n) { return decltype(n)::kBlobBytes; });
    if (!buf) return RAST_OK;
    if (!c->mlp_ready) return fail(c, RAST_ERR_INVALID_ARG, "no trained or loaded weights");
    if (cap < *size) return fail(c, RAST_ERR_INVALID_ARG, "buffer too small for the weight blob");
    return with_mlp_net(net, [&](auto n) {
        using N = decltype(n);
        MlpBlobHeader h;
        std::memset(&h, 0, sizeof h);
        std::memcpy(h.magic, "RMLP", 4);
        h.version = kMlpBlobVersion;
        h.n_in = N::kFeat;
        h.n_hidden = N::kHid;
        h.n_out = kMlpOut;
        h.n_freq = N::kFreq;
        h.n_lights = (uint32_t)c->mlp_nl;
        h.lights_hash = c->mlp_lights_hash;
        h.out_scale = c->mlp_scale;
        h.train_loss = c->mlp_loss;
        unsigned char* o = static_cast<unsigned char*>(buf);
        std::memcpy(o, &h, sizeof h);
        o += sizeof h;
        auto put16 = [&](float f) {
            const uint16_t b = bf16_bits(f);
            std::memcpy(o, &b, 2);
            o += 2;
        };
        const std::vector<float>& q = c->mlp_q;
        for (int r = 0; r < N::kHid; ++r)
            for (int k = 0; k < N::kFeat; ++k) put16(q[N::kPW1 + r * N::kIn + k]);
        for (int i = 0; i < N::kHid * N::kHid; ++i) put16(q[N::kPW2 + i]);
        for (int i = 0; i < kMlpOut * N::kHid; ++i) put16(q[N::kPW3 + i]);
        return RAST_OK;
    });
}

rast_status rast_mlp_load(rast_ctx* c, const void* buf, size_t size) {
    if (!c || !buf) return RAST_ERR_INVALID_ARG;
    if (size < sizeof(MlpBlobHeader)) return fail(c, RAST_ERR_INVALID_ARG, "weight blob has the wrong size");
    MlpBlobHeader h;
    std::memcpy(&h, buf, sizeof h);
    if (std::memcmp(h.magic, "RMLP", 4) != 0 || h.version != kMlpBlobVersion)
        return fail(c, RAST_ERR_INVALID_ARG, "not an RMLP version " + std::to_string(kMlpBlobVersion) + " blob");
    // the network whose dimensions the header gives
    int net = -1;
    for (int cand : {kMlpNetCompact, kMlpNetWide})
        if (with_mlp_net(cand, [&](auto n) {
                using N = decltype(n);
                return h.n_in == (uint32_t)N::kFeat && h.n_hidden == (uint32_t)N::kHid && h.n_out == (uint32_t)kMlpOut &&
                       h.n_freq == (uint32_t)N::kFreq;
            }))
            net = cand;
    if (net < 0 || !(h.out_scale > 0.f)) return fail(c, RAST_ERR_INVALID_ARG, "weight blob has other dimensions");
    if (size != with_mlp_net(net, [](auto n) { return decltype(n)::kBlobBytes; }))
        return fail(c, RAST_ERR_INVALID_ARG, "weight blob has the wrong size");
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    const rast_status st = with_mlp_net(net, [&](auto n) {
        using N = decltype(n);
        const unsigned char* p = static_cast<const unsigned char*>(buf) + sizeof h;
        auto get16 = [&]() {
            uint16_t b;
            std::memcpy(&b, p, 2);
            p += 2;
            return bf16_value(b);
        };
        std::vector<float> q(N::kParams, 0.f);
        for (int r = 0; r < N::kHid; ++r)
            for (int k = 0; k < N::kFeat; ++k) q[N::kPW1 + r * N::kIn + k] = get16();
        for (int i = 0; i < N::kHid * N::kHid; ++i) q[N::kPW2 + i] = get16();
        for (int i = 0; i < kMlpOut * N::kHid; ++i) q[N::kPW3 + i] = get16();
        return install<N>(c, q, h.out_scale, h.train_loss);
    });
    if (st != RAST_OK) return st;
    // the rig the weights belong to, whatever lights are set now
    c->mlp_nl = (int32_t)h.n_lights;
    c->mlp_lights_hash = h.lights_hash;
    return RAST_OK;
}

rast_status rast_mlp_eval(rast_ctx* c, const float* normals3, const float* albedo3, int64_t n, int32_t exact,
                          float* out3) {
    if (!c) return RAST_ERR_INVALID_ARG;
    if (n < 0 || n > ((int64_t)1 << 26) || (n && (!normals3 || !albedo3 || !out3)))
        return fail(c, RAST_ERR_INVALID_ARG, "bad evaluation arguments");
    if (!exact && !c->mlp_ready) return fail(c, RAST_ERR_INVALID_ARG, "no trained or loaded weights");
    if (n == 0) return RAST_OK;
    DeviceGuard g(c->device);
    RAST_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<float> rec(6 * (size_t)n);
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            rec[6 * i + k] = normals3[3 * i + k];
            rec[6 * i + 3 + k] = albedo3[3 * i + k];
        }
    TempBuf src, dst;
    RAST_CUDA(c, src.reserve(sizeof(float) * rec.size()));
    RAST_CUDA(c, dst.reserve(sizeof(float) * 3 * (size_t)n));
    RAST_CUDA(c, cudaMemcpy(src.ptr, rec.data(), sizeof(float) * rec.size(), cudaMemcpyHostToDevice));
    if (!c->lights.ptr) RAST_CUDA(c, c->lights.reserve(sizeof(float) * 7));
    const rast_status st = eval_device(c, src.as<float>(), 6, n, exact != 0, dst.as<float>());
    if (st != RAST_OK) return st;
    RAST_CUDA(c, cudaMemcpy(out3, dst.ptr, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost));
    return RAST_OK;
}

}  // extern "C"
