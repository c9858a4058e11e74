// Instantiations of the fast convolution pass kernels, lengths 280, 288, 320, 336, 300, 324, 384.
#include <vector>

#include "fft_fast.cuh"

namespace pvd {

void fast_lens_part2(std::vector<FastLen>& v) {
  v.push_back(make_fast_len<14, 20>());  // 280
  v.push_back(make_fast_len<16, 18>());  // 288
  v.push_back(make_fast_len<16, 20>());  // 320
  v.push_back(make_fast_len<16, 21>());  // 336
  v.push_back(make_fast_len<15, 20>());  // 300
  v.push_back(make_fast_len<18, 18>());  // 324
  v.push_back(make_fast_len<16, 24>());  // 384
}

}  // namespace pvd
