// Drives the C++ adapters with the reference's call signatures (tests/test_gpu_adapters.py builds
// and runs it).  Reads a float32 field from argv[1] (raw, x fastest) with dims argv[2..4] on
// [-1,1]^3 and an isovalue argv[5]; writes counts and arrays to argv[6] as raw binary.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "../../include/tmc_gb300_adapters.hpp"

int main(int argc, char** argv) {
  if (argc < 8) {
    std::fprintf(stderr, "usage: field.raw nx ny nz iso out.bin volume.ushort\n");
    return 2;
  }
  const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
  const double iso = std::atof(argv[5]);
  std::vector<float> f((size_t)nx * ny * nz);
  std::FILE* in = std::fopen(argv[1], "rb");
  if (!in || std::fread(f.data(), sizeof(float), f.size(), in) != f.size()) return 3;
  std::fclose(in);
  try {
    // cpp_dmc style
    tmc_gb300::dmc::UniformGrid ug;
    tmc_gb300::dmc::UniformGrid::BBox bb;
    for (int c = 0; c < 8; c++) bb[c] = tmc_gb300::dmc::Vector{{(c & 1) ? 1.0 : -1.0, (c & 2) ? 1.0 : -1.0, (c & 4) ? 1.0 : -1.0}};
    ug.init(nx, ny, nz, bb);
    ug.set_dx(2.0 / (nx - 1));
    ug.set_dy(2.0 / (ny - 1));
    ug.set_dz(2.0 / (nz - 1));
    for (size_t s = 0; s < f.size(); s++) ug.scalar((int)s, f[s]);
    tmc_gb300::dmc::DualMarchingCubes dmc;
    std::vector<tmc_gb300::dmc::Vector> v, n;
    std::vector<int> t, q;
    dmc.dualMC(iso, ug, v, n, t, q, true);
    // cuda_tmc style, from a ushort volume file
    tmc_gb300::p_mc::MarchingCubes mc;
    int nr_v = 0, nr_t = 0;
    float *vv = nullptr, *nn = nullptr;
    int* tt = nullptr;
    mc.mc_sharedvertex(1000.0f, argv[7], nr_v, &vv, &nn, nr_t, &tt);
    std::ofstream o(argv[6], std::ios::binary);
    const long long cnt[4] = {(long long)v.size(), (long long)(q.size() / 4), (long long)nr_v, (long long)nr_t};
    o.write((const char*)cnt, sizeof cnt);
    for (auto& p : v) o.write((const char*)p.p, 3 * sizeof(double));
    o.write((const char*)q.data(), q.size() * sizeof(int));
    o.write((const char*)t.data(), t.size() * sizeof(int));
    o.write((const char*)tt, 3 * (size_t)nr_t * sizeof(int));
    o.write((const char*)vv, 3 * (size_t)nr_v * sizeof(float));
    delete[] vv;
    delete[] nn;
    delete[] tt;
  } catch (const tmc_gb300::Error& e) {
    std::fprintf(stderr, "tmc_gb300 error %d: %s\n", (int)e.status, e.what());
    return 1;
  }
  return 0;
}
