/*
 * ref_cpu_harness.cu -- the reference's CPU RoarGraph path as a library
 * (TEST INFRASTRUCTURE ONLY; tests/golden/make_golden_cpu.py is its only user).
 *
 * Built by oracle/build_ref_cpu.sh on an x86-64 host with AVX-512: it includes the reference's
 * own driver tests/test_t2iend.cu where it lies (with oracle/ref_stub/ standing in for spdlog and
 * googletest; the driver's TEST body is compiled but never called) and exports its CPU functions
 * with plain C signatures:
 *   ref_cpu_compare      compare          tests/test_t2iend.cu:31-80 (AVX-512 inner product)
 *   ref_cpu_match_nn_ep  MatchNN's ep     :179-318
 *   ref_cpu_match_sup    MatchSup         :365-488
 *   ref_cpu_fusion_nn    FusionNN         :490-537
 *   ref_cpu_fusion_final FusionFinal      :539-613
 * Every function runs with thread_limit = 1, so the reverse-edge appends of MatchSup
 * (degrees[].fetch_add) happen in ascending query order.  Graphs are exchanged as CSR
 * (off[n + 1], ids[off[n]]).
 */
#include "test_t2iend.cu"

#include <cstring>

namespace {
using Lists = std::vector<std::vector<uint32_t>>;

Lists from_csr(uint32_t n, const uint64_t* off, const uint32_t* ids) {
  Lists g(n);
  for (uint32_t i = 0; i < n; i++) g[i].assign(ids + off[i], ids + off[i + 1]);
  return g;
}

// Writes g as CSR; returns the number of ids, or -1 when cap is too small.
long long to_csr(const Lists& g, uint64_t* off, uint32_t* ids, uint64_t cap) {
  uint64_t o = 0;
  for (size_t i = 0; i < g.size(); i++) {
    off[i] = o;
    if (o + g[i].size() > cap) return -1;
    std::memcpy(ids + o, g[i].data(), g[i].size() * 4);
    o += g[i].size();
  }
  off[g.size()] = o;
  return static_cast<long long>(o);
}
}  // namespace

extern "C" {

float ref_cpu_compare(const float* a, const float* b, uint32_t d) {
  return Gbuilder::Gpu::compare(a, b, d);
}

uint32_t ref_cpu_match_nn_ep(uint32_t n, uint32_t q, const uint32_t* gt, const float* data,
                             uint32_t d) {
  uint32_t ep = 0;
  Gbuilder::Gpu::MatchNN(n, q, 128, 128, 40, gt, ep, data, d, 1);
  return ep;
}

long long ref_cpu_match_sup(uint32_t n, uint32_t q, uint32_t topn, uint32_t n_ctr, uint32_t m_nn,
                            const uint32_t* gt, const float* data, uint32_t d, uint64_t* off,
                            uint32_t* ids, uint64_t cap) {
  Lists g = Gbuilder::Gpu::MatchSup(n, q, topn, n_ctr, m_nn, gt, data, d, 1);
  return to_csr(g, off, ids, cap);
}

// supply: `rounds` CSR graphs back to back (offsets (n + 1) each, ids concatenated with
// supply_base[r] the start of round r's ids)
long long ref_cpu_fusion_nn(uint32_t n, uint32_t m_nn, const float* data, uint32_t d,
                            uint32_t rounds, const uint64_t* supply_off,
                            const uint32_t* supply_ids, const uint64_t* supply_base,
                            uint64_t* off, uint32_t* ids, uint64_t cap) {
  Lists top(n);
  std::vector<Lists> sup;
  for (uint32_t r = 0; r < rounds; r++)
    sup.push_back(from_csr(n, supply_off + static_cast<uint64_t>(r) * (n + 1),
                           supply_ids + supply_base[r]));
  Lists g = Gbuilder::Gpu::FusionNN(n, m_nn, data, top, sup, d, 1);
  return to_csr(g, off, ids, cap);
}

long long ref_cpu_fusion_final(uint32_t n, uint32_t m_supply, uint32_t m_link, uint32_t m_final,
                               const float* data, uint32_t d, const uint32_t* supply,
                               const uint64_t* bip_off, const uint32_t* bip_ids,
                               const uint32_t* link, uint64_t* off, uint32_t* ids, uint64_t cap) {
  std::vector<uint32_t> sup(supply, supply + static_cast<uint64_t>(n) * m_supply);
  std::vector<uint32_t> lnk(link, link + static_cast<uint64_t>(n) * m_link);
  Lists bip = from_csr(n, bip_off, bip_ids);
  Lists g = Gbuilder::Gpu::FusionFinal(n, m_supply, m_link, m_final, data, sup, bip, lnk, d, 1);
  return to_csr(g, off, ids, cap);
}

}  // extern "C"
