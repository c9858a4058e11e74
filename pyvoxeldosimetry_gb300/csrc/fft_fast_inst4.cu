// Instantiations of the fast convolution pass kernels, lengths 560, 576, 640.
#include <vector>

#include "fft_fast.cuh"

namespace pvd {

void fast_lens_part4(std::vector<FastLen>& v) {
  v.push_back(make_fast_len<20, 28>());  // 560
  v.push_back(make_fast_len<24, 24>());  // 576
  v.push_back(make_fast_len<20, 32>());  // 640
}

}  // namespace pvd
