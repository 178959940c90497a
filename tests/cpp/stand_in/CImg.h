// Test stand-in for the slice of CImg the drop-in uses: an image of width x height x depth x
// spectrum values stored plane by plane (x + y*W + z*W*H + c*W*H*D), with data(), width(),
// height() and spectrum().
#ifndef RAST_TEST_CIMG_STAND_IN_H
#define RAST_TEST_CIMG_STAND_IN_H
#include <vector>
namespace cimg_library {
template <typename T>
class CImg {
    std::vector<T> buf_;
    unsigned w_, h_, d_, s_;
public:
    CImg() : w_(0), h_(0), d_(0), s_(0) {}
    CImg(unsigned w, unsigned h, unsigned d, unsigned s, const T& value)
        : buf_((size_t)w * h * d * s, value), w_(w), h_(h), d_(d), s_(s) {}
    T* data() { return buf_.data(); }
    const T* data() const { return buf_.data(); }
    int width() const { return (int)w_; }
    int height() const { return (int)h_; }
    int depth() const { return (int)d_; }
    int spectrum() const { return (int)s_; }
};
}  // namespace cimg_library
#endif
