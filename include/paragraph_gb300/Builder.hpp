// Builder.hpp -- Gbuilder::Builder<T>, header-only, over the C ABI of paragraph_gb300.h.
//
// The reference declares this class (include/Builder.hpp:15-35) but ships it commented out, and
// src/Builder.cpp is empty; its driver launches the kernel templates directly
// (tests/test_t2iend.cu:974-1139).  This restores the declared interface -- construction from
// base vectors and ground-truth ids, SetGt, LaunchBuild -- on top of libparagraph_gb300.so, adds
// LaunchIndex for the driver's whole index (the file the driver saves), with
// sizes as runtime values.  LaunchBuild's template arguments are kept for source compatibility:
// grid_size/block_size are ignored (the library chooses launch shapes), gt_num and dim are
// checked against the data.  Errors throw Gbuilder::BuildError carrying the pg_status code.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../paragraph_gb300.h"

namespace Gbuilder {

class BuildError : public std::runtime_error {
 public:
  BuildError(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != PG_OK) throw BuildError(rc, pg_last_error());
}

template <typename T>
class Builder {
  static_assert(sizeof(T) == 4, "the GPU build path computes on float32 vectors");

 public:
  using data_type = T;
  using id_type = uint32_t;

  Builder() = delete;

  // base: n x dim row-major; gt_ids: q x gt_num row-major (tomb-padded, as
  // transform_gt_to_128.ipynb writes it).  `dim` is needed because a flat vector has no shape.
  Builder(std::vector<data_type> const& base, std::vector<id_type> const& gt_ids, uint32_t dim,
          uint32_t degree = 32, uint32_t beam = 64, int device = 0)
      : base_(base), gt_ids_(gt_ids), dim_(dim), device_(device) {
    check(pg_params_default(&params_, degree, beam));
  }

  Builder(Builder&& other) noexcept
      : base_(std::move(other.base_)),
        gt_ids_(std::move(other.gt_ids_)),
        dim_(other.dim_),
        device_(other.device_),
        params_(other.params_),
        graph_(std::move(other.graph_)),
        projection_(std::move(other.projection_)),
        index_(std::move(other.index_)),
        index_stride_(other.index_stride_),
        stats_(other.stats_),
        ep_(other.ep_) {}
  Builder(Builder& other) = delete;
  Builder& operator=(Builder const&) = delete;
  Builder& operator=(Builder&&) = delete;
  ~Builder() = default;

  // Runs the whole GPU build (projection + link rounds); the result is graph() (n x degree,
  // tomb padded), projection() (n x 16) and ep().
  template <uint32_t grid_size, uint32_t block_size, uint32_t gt_num, uint32_t dim>
  auto LaunchBuild() -> void {
    if (dim != dim_) throw BuildError(PG_EINVAL, "LaunchBuild: dim differs from the data");
    if (gt_num != params_.gt_k) throw BuildError(PG_EINVAL, "LaunchBuild: gt_num != gt_k");
    LaunchBuild();
  }

  auto LaunchBuild() -> void {
    if (dim_ == 0 || base_.size() % dim_ != 0) throw BuildError(PG_EINVAL, "base size % dim");
    if (gt_ids_.size() % params_.gt_k != 0) throw BuildError(PG_EINVAL, "gt size % gt_k");
    const uint64_t n = base_.size() / dim_;
    const uint64_t q = gt_ids_.size() / params_.gt_k;
    graph_.assign(n * params_.degree, PG_TOMB);
    projection_.assign(n * params_.proj_degree, PG_TOMB);
    index_.clear();
    index_stride_ = 0;
    pg_handle h = nullptr;
    check(pg_create(&h, device_, nullptr));
    const int rc = pg_build_host(h, &params_, reinterpret_cast<const float*>(base_.data()), n,
                                 dim_, gt_ids_.data(), q, graph_.data(), projection_.data(),
                                 &stats_);
    pg_destroy(h);
    check(rc);
    check(pg_entry_point(gt_ids_.data(), q, params_.gt_k, n, &ep_));
  }

  // The reference driver's whole index (tests/test_t2iend.cu:974-1258): the GPU build, then
  // `match_rounds` MatchSup rounds, FusionNN(m_nn) and FusionFinal(m_final), on the GPU
  // (pg_build_index_host).  The driver's values are 6, 40 and 70.  The result is index() (n rows
  // of 2*m_nn + m_final slots, tomb padded), which SaveGraph then writes, as the driver saves its
  // FusionFinal graph.
  auto LaunchIndex(uint32_t match_rounds = 6, uint32_t m_nn = 40, uint32_t m_final = 70) -> void {
    if (dim_ == 0 || base_.size() % dim_ != 0) throw BuildError(PG_EINVAL, "base size % dim");
    if (gt_ids_.size() % params_.gt_k != 0) throw BuildError(PG_EINVAL, "gt size % gt_k");
    const uint64_t n = base_.size() / dim_;
    const uint64_t q = gt_ids_.size() / params_.gt_k;
    const uint32_t stride = 2 * m_nn + m_final;
    std::vector<id_type> rows(n * stride);
    std::vector<uint32_t> cnt(n);
    pg_handle h = nullptr;
    check(pg_create(&h, device_, nullptr));
    const int rc = pg_build_index_host(h, &params_, reinterpret_cast<const float*>(base_.data()),
                                       n, dim_, gt_ids_.data(), q, match_rounds, m_nn, m_final,
                                       stride, rows.data(), cnt.data(), &stats_);
    pg_destroy(h);
    check(rc);
    for (uint64_t i = 0; i < n; i++)
      for (uint32_t j = cnt[i]; j < stride; j++) rows[i * stride + j] = PG_TOMB;
    index_ = std::move(rows);
    index_stride_ = stride;
    check(pg_entry_point(gt_ids_.data(), q, params_.gt_k, n, &ep_));
  }

  auto SetGt(std::vector<id_type>&& gt_ids) -> void { gt_ids_ = std::move(gt_ids); }

  // SaveGraph (tests/test_t2iend.cu:615-633): the FusionFinal index when LaunchIndex has run
  // (what the reference driver saves, :1258), else the graph of LaunchBuild.
  auto SaveGraph(std::string const& path) const -> void {
    if (index_stride_) {
      check(pg_save_graph(path.c_str(), index_.data(), index_.size() / index_stride_,
                          index_stride_, ep_));
      return;
    }
    check(pg_save_graph(path.c_str(), graph_.data(), graph_.size() / params_.degree,
                        params_.degree, ep_));
  }

  pg_params& params() { return params_; }
  std::vector<id_type> const& graph() const { return graph_; }
  std::vector<id_type> const& projection() const { return projection_; }
  std::vector<id_type> const& index() const { return index_; }
  uint32_t index_stride() const { return index_stride_; }
  pg_stats const& stats() const { return stats_; }
  id_type ep() const { return ep_; }

 private:
  std::vector<data_type> base_;
  std::vector<id_type> gt_ids_;
  uint32_t dim_ = 0;
  int device_ = 0;
  pg_params params_{};
  std::vector<id_type> graph_;
  std::vector<id_type> projection_;
  std::vector<id_type> index_;
  uint32_t index_stride_ = 0;
  pg_stats stats_{};
  id_type ep_ = 0;
};

}  // namespace Gbuilder
