// Host build of csrc/exact_pred.cuh for the CPU tests: reads m groups of four
// float32 planes (16 floats each) and writes, per group, the signs of det4,
// det3 of the first three normals, and exact_side (three int32).
//
//   exact_pred_host <rows.f32> <m> <out.i32>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "exact_pred.cuh"

using namespace vgb;

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  const int m = std::atoi(argv[2]);
  std::vector<float> v((size_t)m * 16);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(v.data(), sizeof(float), v.size(), f) != v.size()) return 3;
  std::fclose(f);
  std::vector<int> out((size_t)m * 3);
  for (int g = 0; g < m; ++g) {
    float4 r[4];
    for (int i = 0; i < 4; ++i) {
      const float* p = &v[(size_t)g * 16 + 4 * i];
      r[i] = make_float4(p[0], p[1], p[2], p[3]);
    }
    out[3 * g] = exact_det4_sign(r[0], r[1], r[2], r[3]);
    out[3 * g + 1] = exact_det3_sign(r[0], r[1], r[2]);
    out[3 * g + 2] = exact_side(r[0], r[1], r[2], r[3]);
  }
  f = std::fopen(argv[3], "wb");
  if (!f || std::fwrite(out.data(), sizeof(int), out.size(), f) != out.size()) return 4;
  std::fclose(f);
  return 0;
}
