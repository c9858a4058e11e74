// Registry of the fast FFT lengths instantiated in fft_fast_inst*.cu.
#include <algorithm>
#include <vector>

#include "../../include/pvd.h"
#include "fft_fast.cuh"

namespace pvd {

void fast_lens_part0(std::vector<FastLen>& v);
void fast_lens_part1(std::vector<FastLen>& v);
void fast_lens_part2(std::vector<FastLen>& v);
void fast_lens_part3(std::vector<FastLen>& v);
void fast_lens_part4(std::vector<FastLen>& v);

static const std::vector<FastLen>& fast_table() {
  static const std::vector<FastLen> t = [] {
    std::vector<FastLen> v;
    fast_lens_part0(v);
    fast_lens_part1(v);
    fast_lens_part2(v);
    fast_lens_part3(v);
    fast_lens_part4(v);
    std::sort(v.begin(), v.end(), [](const FastLen& a, const FastLen& b) { return a.L < b.L; });
    return v;
  }();
  return t;
}

const FastLen* fast_len(int L) {
  for (const FastLen& f : fast_table())
    if (f.L == L) return &f;
  return nullptr;
}

int fast_len_at_least(int n) {
  for (const FastLen& f : fast_table())
    if (f.L >= n) return f.L;
  return 0;
}

}  // namespace pvd

extern "C" int pvd_fast_lengths(int* out, int cap) {
  const auto& t = pvd::fast_table();
  int n = 0;
  for (const auto& f : t) {
    if (out && n < cap) out[n] = f.L;
    ++n;
  }
  return n;
}
