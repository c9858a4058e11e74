// Instantiations of the fast convolution pass kernels, lengths 360, 400, 448, 512, 480.
#include <vector>

#include "fft_fast.cuh"

namespace pvd {

void fast_lens_part3(std::vector<FastLen>& v) {
  v.push_back(make_fast_len<18, 20>());  // 360
  v.push_back(make_fast_len<20, 20>());  // 400
  v.push_back(make_fast_len<16, 28>());  // 448
  v.push_back(make_fast_len<16, 32>());  // 512
  v.push_back(make_fast_len<20, 24>());  // 480
}

}  // namespace pvd
