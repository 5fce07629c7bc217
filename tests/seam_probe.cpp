// Uses the C++ mirror of the reference seam (host/hausdorff_distance.h) the
// way the reference's driver does, for tests/test_hd_exec_gpu.py.
// usage: seam_probe <A.bin> <B.bin>   (3-D points)
#include <cstdio>
#include <vector>

#include "hausdorff_distance.h"
#include "loaders.h"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  hd::PointSet a = hd::LoadBin(argv[1], 3, 1u << 30), b = hd::LoadBin(argv[2], 3, 1u << 30);
  std::vector<hd::Point<3>> va(a.size()), vb(b.size());
  for (size_t i = 0; i < a.size(); ++i)
    for (int k = 0; k < 3; ++k) va[i].c[k] = a.xyz[i * 3 + k];
  for (size_t i = 0; i < b.size(); ++i)
    for (int k = 0; k < 3; ++k) vb[i].c[k] = b.xyz[i * 3 + k];
  hd::HausdorffDistanceEarlyBreak<float, 3> eb;
  hd::HausdorffDistanceHybrid<float, 3> hy;
  hd::HausdorffDistanceRayTracing<float, 3> rt;
  const float d1 = eb.CalculateDistance(va, vb);
  const float d2 = hy.CalculateDistance(va, vb);
  const float d3 = rt.CalculateDistance(va, vb);
  std::printf("%.9g %.9g %.9g\n", d1, d2, d3);
  std::printf("%s\n", rt.get_stats().dump(0).c_str());
  // The double instantiation (hd_solve_f64) on the same points.
  std::vector<hd::Point<3, double>> wa(a.size()), wb(b.size());
  for (size_t i = 0; i < a.size(); ++i)
    for (int k = 0; k < 3; ++k) wa[i].c[k] = a.xyz[i * 3 + k];
  for (size_t i = 0; i < b.size(); ++i)
    for (int k = 0; k < 3; ++k) wb[i].c[k] = b.xyz[i * 3 + k];
  hd::HausdorffDistanceHybrid<double, 3> hy64;
  try {
    std::vector<hd::Point<3>> empty;
    eb.CalculateDistance(empty, vb);
  } catch (const hd::Error& e) {
    std::printf("error %d\n", (int) e.status);
  }
  std::printf("%.17g\n", hy64.CalculateDistance(wa, wb));
  return 0;
}
