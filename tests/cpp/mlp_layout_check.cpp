// Host-side checks of the learned shader's two networks (rasteriser_gb300/csrc/rast_mlp.h): the
// sizes and offsets of the device image, the parameters the optimiser keeps fixed, and the
// tensor-core operand layout (core_offset), which must place every element of W1, W2 and W3 at
// its own 2-byte slot inside the operand. Prints "ok" and exits 0, or names the first failure.
#include <cstdio>
#include <vector>

#include "rast_mlp.h"

using namespace rast;

static int fails = 0;
#define CHECK(c)                                                            \
    do {                                                                    \
        if (!(c)) {                                                         \
            std::printf("failed: %s (line %d)\n", #c, __LINE__);            \
            ++fails;                                                        \
        }                                                                   \
    } while (0)

// Every (row, k) of a rows x K operand at a distinct, in-range, 2-byte-aligned offset.
static void check_operand(uint32_t rows, uint32_t K) {
    std::vector<int> seen(rows * K, 0);
    for (uint32_t r = 0; r < rows; ++r)
        for (uint32_t k = 0; k < K; ++k) {
            const uint32_t off = core_offset(rows, r, k);
            CHECK(off % 2 == 0 && off / 2 < rows * K);
            if (off / 2 < rows * K) ++seen[off / 2];
        }
    for (int s : seen) CHECK(s == 1);
}

template <class N>
static void check_net(int freq, int hid) {
    CHECK(N::kFreq == freq && N::kHid == hid);
    CHECK(N::kFeat == 6 * freq + 7 && N::kConst == N::kFeat - 1 && N::kIn >= N::kFeat && N::kIn % 16 == 0);
    CHECK(N::kUnit1 == hid - 1);
    CHECK(N::kPW2 == hid * N::kIn && N::kPW3 == N::kPW2 + hid * hid && N::kParams == N::kPW3 + kMlpOut * hid);
    CHECK(N::kW2Off == 2u * hid * N::kIn && N::kW3Off == N::kW2Off + 2u * hid * hid);
    CHECK(N::kScaleOff == N::kW3Off + 2u * kMlpOutPad * hid && N::kImageBytes == N::kScaleOff + 16u);
    CHECK(N::kImageBytes % 16 == 0);
    CHECK(N::kBlobBytes == sizeof(MlpBlobHeader) + 2 * (hid * N::kFeat + hid * hid + kMlpOut * hid));
    // fixed parameters: W1's padding columns and W1's / W2's constant rows, nothing else
    int fixed = 0;
    for (int p = 0; p < N::kParams; ++p) {
        bool want = false;
        if (p < N::kPW2) want = (p % N::kIn) >= N::kFeat || p / N::kIn == N::kUnit1;
        else if (p < N::kPW3) want = (p - N::kPW2) / hid == N::kUnit1;
        CHECK(N::fixed(p) == want);
        fixed += N::fixed(p) ? 1 : 0;
    }
    const int want_fixed = hid * (N::kIn - N::kFeat) + N::kFeat + hid;
    CHECK(fixed == want_fixed);
    check_operand(hid, N::kIn);
    check_operand(hid, hid);
    check_operand(kMlpOutPad, hid);
}

int main() {
    check_net<MlpCompact>(3, 32);
    check_net<MlpWide>(16, 64);
    CHECK(MlpCompact::kIn == 32 && MlpWide::kIn == 112);
    CHECK(sizeof(MlpCheckTable) == 24u * kMlpCheckLights);
    if (fails) return 1;
    std::printf("ok\n");
    return 0;
}
