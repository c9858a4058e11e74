// Instantiations of the fast convolution pass kernels, lengths 160, 192, 224, 240, 256, 252, 270.
#include <vector>

#include "fft_fast.cuh"

namespace pvd {

void fast_lens_part1(std::vector<FastLen>& v) {
  v.push_back(make_fast_len<10, 16>());  // 160
  v.push_back(make_fast_len<12, 16>());  // 192
  v.push_back(make_fast_len<14, 16>());  // 224
  v.push_back(make_fast_len<15, 16>());  // 240
  v.push_back(make_fast_len<16, 16>());  // 256
  v.push_back(make_fast_len<14, 18>());  // 252
  v.push_back(make_fast_len<15, 18>());  // 270
}

}  // namespace pvd
