// Builds a graph through the restored Gbuilder::Builder<float> (include/paragraph_gb300/Builder.hpp)
// and writes it with SaveGraph, the way a ParaGraph driver would use the class.
// usage: builder_demo BASE_F32 GT_U32 N D DEGREE BEAM OUT_GRAPH [index]
// BASE_F32 / GT_U32 are headerless row-major files (read_vec_from_file's layout, gt top-128).
// With `index`, LaunchIndex builds the driver's whole index and SaveGraph writes it.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "paragraph_gb300/Builder.hpp"

int main(int argc, char** argv) {
  if (argc != 8 && argc != 9) {
    std::fprintf(stderr, "usage: %s BASE GT N D DEGREE BEAM OUT [index]\n", argv[0]);
    return 2;
  }
  const bool index = argc == 9 && std::strcmp(argv[8], "index") == 0;
  const uint64_t n = std::strtoull(argv[3], nullptr, 10);
  const uint32_t d = static_cast<uint32_t>(std::strtoul(argv[4], nullptr, 10));
  const uint32_t degree = static_cast<uint32_t>(std::strtoul(argv[5], nullptr, 10));
  const uint32_t beam = static_cast<uint32_t>(std::strtoul(argv[6], nullptr, 10));
  std::vector<float> base(n * d);
  std::vector<uint32_t> gt(n * 128);
  try {
    Gbuilder::check(pg_read_file(argv[1], 0, base.data(), base.size() * 4, nullptr, nullptr));
    Gbuilder::check(pg_read_file(argv[2], 0, gt.data(), gt.size() * 4, nullptr, nullptr));
    Gbuilder::Builder<float> b(base, gt, d, degree, beam);
    if (index)
      b.LaunchIndex();
    else
      b.LaunchBuild();
    b.SaveGraph(argv[7]);
    std::printf("ep %u evals %llu\n", b.ep(),
                static_cast<unsigned long long>(b.stats().evals_total));
  } catch (Gbuilder::BuildError const& e) {
    std::fprintf(stderr, "build failed (%d): %s\n", e.code(), e.what());
    return 1;
  }
  return 0;
}
