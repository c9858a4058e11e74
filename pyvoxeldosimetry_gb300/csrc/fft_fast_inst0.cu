// Instantiations of the fast convolution pass kernels, lengths 64, 72, 80, 96, 112, 128, 144.
#include <vector>

#include "fft_fast.cuh"

namespace pvd {

void fast_lens_part0(std::vector<FastLen>& v) {
  v.push_back(make_fast_len<8, 8>());  // 64
  v.push_back(make_fast_len<8, 9>());  // 72
  v.push_back(make_fast_len<8, 10>());  // 80
  v.push_back(make_fast_len<8, 12>());  // 96
  v.push_back(make_fast_len<8, 14>());  // 112
  v.push_back(make_fast_len<8, 16>());  // 128
  v.push_back(make_fast_len<12, 12>());  // 144
}

}  // namespace pvd
