// mkf_gb300.hpp -- C++ classes over the C ABI of libmkf_gb300.so, shaped like
// the reference's own classes so that a C++ caller (the reference's PFTracker,
// or the standalone harness that replaces it) keeps its construct / load /
// reset / update / estimate call sequence:
//
//   reference (OpenCV + ROS)                       here
//   pf2DRao ParticleFilter(int)  pf2DRao.h:13-31    mkf::RaoParticleFilter
//     .gmm.loadGaussian(u, s, H, m, w, g)           .gmm.loadGaussian(...)
//     .gmm.resetTracker(bins)  my_gmm.h:20-33       .gmm.resetTracker(bins)
//     .resample(w, N)          pf2DRao.cpp:175      mkf::resample(w, N, U)
//     .update(measurement)     pf2DRao.cpp:125      .update(d_meas, mask, frame)
//     .getEstimator()          pf2DRao.cpp:23       .getEstimator()
//   pf2D ParticleFilter(N, d, side) pf2D.h:25-51    mkf::LegacyParticleFilter
//   PFTracker::getMeasurementProposal + update      mkf::PoseTracker::stepImage (likelihood
//     (pfPose.cpp:210-329, 332-385)                  image) / ::step (detection list)
//   get3Dpose / publish2Dpos (pfPose.cpp:93-208)     mkf::PoseDecoder
//   (no counterpart: one tracker per arm)            mkf::BatchedBootstrapPF (thousands of
//                                                      uneven tracks in one persistent launch)
//
// Errors: every non-MKF_OK status becomes an mkf::Error carrying the status and
// mkf_last_error().  Handles are move-only RAII owners.  Device buffers are
// mkf::DeviceArray<T>.  A filter object is single-stream and not thread-safe
// (as the reference's were); distinct objects are independent.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mkf_gb300.h"

namespace mkf {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status(status) {}
  int status;
};

inline void check(int status, const char* what) {
  if (status != MKF_OK) {
    const char* msg = mkf_last_error();
    throw Error(status, std::string(what) + ": " + (msg ? msg : ""));
  }
}

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(MKF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
class DeviceArray {
 public:
  DeviceArray() = default;
  explicit DeviceArray(size_t n) : n_(n) {
    if (n) cuda_check(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(T)), "cudaMalloc");
  }
  DeviceArray(const T* host, size_t n) : DeviceArray(n) { upload(host, n); }
  explicit DeviceArray(const std::vector<T>& v) : DeviceArray(v.data(), v.size()) {}
  ~DeviceArray() { if (p_) cudaFree(p_); }
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  DeviceArray(DeviceArray&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
  DeviceArray& operator=(DeviceArray&& o) noexcept {
    if (this != &o) { if (p_) cudaFree(p_); p_ = o.p_; n_ = o.n_; o.p_ = nullptr; o.n_ = 0; }
    return *this;
  }
  T* data() { return p_; }
  const T* data() const { return p_; }
  size_t size() const { return n_; }
  void upload(const T* host, size_t n, cudaStream_t s = nullptr) {
    if (n > n_) throw Error(MKF_ERR_ARG, "DeviceArray::upload: too many elements");
    if (n) cuda_check(cudaMemcpyAsync(p_, host, n * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
  }
  void download(T* host, size_t n, cudaStream_t s = nullptr) const {
    if (n > n_) throw Error(MKF_ERR_ARG, "DeviceArray::download: too many elements");
    if (n) cuda_check(cudaMemcpyAsync(host, p_, n * sizeof(T), cudaMemcpyDeviceToHost, s), "download");
    cuda_check(cudaStreamSynchronize(s), "download sync");
  }
  std::vector<T> to_host(cudaStream_t s = nullptr) const {
    std::vector<T> v(n_);
    download(v.data(), n_, s);
    return v;
  }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
};

// ParticleFilter::resample (pf2DRao.cpp:175-210) with an explicit 32-bit
// uniform U (U / 2^32 in [0, 1)): N ancestors of the L weights in w.
inline std::vector<int> resample(const std::vector<double>& w, int N, uint32_t U, cudaStream_t s = nullptr) {
  DeviceArray<double> dw(w);
  DeviceArray<int> idx(static_cast<size_t>(N));
  check(mkf_resample_f64(dw.data(), static_cast<int>(w.size()), N, U, idx.data(), nullptr, s), "mkf_resample_f64");
  return idx.to_host(s);
}

// The reference node's hard-coded settings in one place (defaults = the
// reference's values): particles per arm (pfPose.cpp:57), candidates per
// particle (216), Pa (247), clutter floor (261, 282), image size (pf2D.cpp:49-50)
// and the Kinect intrinsics of get3Dpose (pfPose.cpp:101).  The blur (15 x 15,
// sigma 3), proposal spread (0.8 w) and R = 100 I are fixed in the kernels.
struct TrackerConfig {
  int particles = 500;
  int candidates_per_particle = 10;
  double Pa = 0.05;
  double clutter = 1e-4;
  int width = 640, height = 480;
  double K[9] = {525.0, 0.0, 319.5, 0.0, 525.0, 239.5, 0.0, 0.0, 1.0};
  uint64_t seed = 0;
};

// ------------------------------------------------------ pf2DRao::ParticleFilter
class RaoParticleFilter {
 public:
  // my_gmm, the filter's public member (my_gmm.h:20-33)
  class Gmm {
   public:
    // my_gmm::loadGaussian(u, s, H, m, w, g) (my_gmm.cpp:45-75): u (d), s (d*d),
    // Hpca (d*F, pca_proj), mpca (F, pca_mean), weight w, mean reversion g
    void loadGaussian(int k, const std::vector<double>& u, const std::vector<double>& s,
                      const std::vector<double>& Hpca, const std::vector<double>& mpca, double w, double g) {
      const int F = static_cast<int>(mpca.size());
      check(mkf_rbpf_load_gaussian(pf_->h_, k, u.data(), s.data(), Hpca.data(), mpca.data(), F, w, g),
            "mkf_rbpf_load_gaussian");
    }
    // my_gmm::resetTracker(bins) (my_gmm.cpp:30-42)
    void resetTracker(const std::vector<int>& bins) {
      check(mkf_rbpf_reset(pf_->h_, bins.data(), pf_->stream_), "mkf_rbpf_reset");
    }
    // bins = resample(weight, N) drawn from the filter's own Philox stream
    void resetTracker() { check(mkf_rbpf_reset(pf_->h_, nullptr, pf_->stream_), "mkf_rbpf_reset"); }

   private:
    friend class RaoParticleFilter;
    RaoParticleFilter* pf_ = nullptr;
  };

  RaoParticleFilter(int nParticles, int d = 12, int m = 6, int K = 15, int meas_mode = MKF_MEAS_LINEAR,
                    uint64_t seed = 0, uint32_t track_id = 0, cudaStream_t stream = nullptr)
      : nParticles(nParticles), d(d), m(m), K(K), stream_(stream), est_(static_cast<size_t>(d)) {
    check(mkf_rbpf_create(d, m, K, nParticles, meas_mode, seed, track_id, &h_), "mkf_rbpf_create");
    gmm.pf_ = this;
  }
  ~RaoParticleFilter() { if (h_) mkf_rbpf_destroy(h_); }
  RaoParticleFilter(const RaoParticleFilter&) = delete;
  RaoParticleFilter& operator=(const RaoParticleFilter&) = delete;

  // hand pixel decode for the PDAF association: rows 0,1 of Hpca^T x + mpca
  void setHandDecode(const std::vector<double>& Hd, const std::vector<double>& hb) {
    check(mkf_rbpf_set_hand_decode(h_, Hd.data(), hb.data(), 1), "mkf_rbpf_set_hand_decode");
  }
  // ParticleFilter::update(measurement) (pf2DRao.cpp:125-158): d_measurement is
  // nParticles rows of m values on the device; mask selects the rows used
  void update(const double* d_measurement, unsigned mask, uint32_t frame) {
    check(mkf_rbpf_update(h_, frame, d_measurement, mask, stream_), "mkf_rbpf_update");
  }
  // getEstimator() (pf2DRao.cpp:23-31), left on the device
  const double* estimatorDevice() {
    check(mkf_rbpf_estimate(h_, est_.data(), stream_), "mkf_rbpf_estimate");
    return est_.data();
  }
  std::vector<double> getEstimator() {
    estimatorDevice();
    return est_.to_host(stream_);
  }
  // the estimate into a caller device buffer of d doubles
  void estimateInto(double* d_out) { check(mkf_rbpf_estimate(h_, d_out, stream_), "mkf_rbpf_estimate"); }
  int status() const {
    int s = 0;
    check(mkf_rbpf_status(h_, &s), "mkf_rbpf_status");
    return s;
  }
  mkf_rbpf_t handle() const { return h_; }
  cudaStream_t stream() const { return stream_; }

  Gmm gmm;
  const int nParticles, d, m, K;

 private:
  mkf_rbpf_t h_ = nullptr;
  cudaStream_t stream_;
  DeviceArray<double> est_;
};

// --------------------------------------------------------- pf2D::ParticleFilter
class LegacyParticleFilter {
 public:
  // ParticleFilter(numParticles, numDims, side) with its my_gmm prior: mean
  // (K*d), cov (K*d*d), w (K)
  LegacyParticleFilter(int numParticles, int numDims, bool side, const std::vector<double>& mean,
                       const std::vector<double>& cov, const std::vector<double>& w, int width = 640,
                       int height = 480, uint64_t seed = 0, uint32_t track_id = 0, cudaStream_t stream = nullptr)
      : N(numParticles), d(numDims), stream_(stream), est_(static_cast<size_t>(numDims)) {
    check(mkf_pf2d_create(numParticles, numDims, side ? 1 : 0, static_cast<int>(w.size()), mean.data(),
                          cov.data(), w.data(), width, height, seed, track_id, &h_),
          "mkf_pf2d_create");
  }
  ~LegacyParticleFilter() { if (h_) mkf_pf2d_destroy(h_); }
  LegacyParticleFilter(const LegacyParticleFilter&) = delete;
  LegacyParticleFilter& operator=(const LegacyParticleFilter&) = delete;
  // update(measurement): z = {head x, head y, hand x, hand y}; the reference's
  // predict() runs inside (after resampling, pf2D.cpp:90-102)
  void update(const double z[4], uint32_t frame) { check(mkf_pf2d_update(h_, frame, z, stream_), "mkf_pf2d_update"); }
  std::vector<double> getEstimator() {
    check(mkf_pf2d_estimate(h_, est_.data(), stream_), "mkf_pf2d_estimate");
    return est_.to_host(stream_);
  }
  const int N, d;

 private:
  mkf_pf2d_t h_ = nullptr;
  cudaStream_t stream_;
  DeviceArray<double> est_;
};

// ------------------------------------------------- PFTracker's frame flow, ROS-free
class PoseTracker {
 public:
  PoseTracker(RaoParticleFilter& arm1, RaoParticleFilter& arm2, double Pa = 0.05, double clutter = 1e-4)
      : a1_(arm1), a2_(arm2), Pa_(Pa), clutter_(clutter),
        meas1_(static_cast<size_t>(arm1.nParticles) * arm1.m), meas2_(static_cast<size_t>(arm2.nParticles) * arm2.m),
        cand_(256) {}

  // One frame (pfPose.cpp:332-385): with a face ROI, associate the hand
  // candidates (PDAF, pfPose.cpp:210-329) and update both arms; without one the
  // frame is skipped (pfPose.cpp:370-378) and false is returned.  roi: 8 doubles
  // (x_offset, y_offset, width, height per arm) or nullptr; cand: M (x, y) pairs.
  // The reference's own frame (pfPose.cpp:332-385, 210-329): blur the MONO8
  // likelihood (device, row pitch in bytes), propose nCand candidates per arm
  // (10 N when 0; uniform in the box below the face on the first frame after a
  // start or a no-face frame, else around the decoded hands), weight by the
  // likelihood over the PDA normaliser, resample and update both arms.
  bool stepImage(uint32_t frame, const double* roi, const uint8_t* d_likelihood, int width, int height, int pitch,
                 int nCand = 0) {
    if (!roi) { init_ = false; return false; }
    if (blur_.size() < static_cast<size_t>(width) * height) blur_ = DeviceArray<uint8_t>(static_cast<size_t>(width) * height);
    check(mkf_likelihood_blur(d_likelihood, width, height, pitch, blur_.data(), width, a1_.stream()),
          "mkf_likelihood_blur");
    const int M = nCand > 0 ? nCand : 10 * a1_.nParticles;
    check(mkf_pdaf_propose_image(a1_.handle(), a2_.handle(), frame, roi, blur_.data(), width, height, width, M,
                                 init_ ? 0 : 1, Pa_, clutter_, meas1_.data(), meas2_.data(), nullptr, nullptr,
                                 nullptr, nullptr, a1_.stream()),
          "mkf_pdaf_propose_image");
    init_ = true;
    a1_.update(meas1_.data(), (1u << a1_.m) - 1u, frame);
    a2_.update(meas2_.data(), (1u << a2_.m) - 1u, frame);
    return true;
  }

  bool step(uint32_t frame, const double* roi, const std::vector<double>& cand) {
    if (!roi) return false;
    const int M = static_cast<int>(cand.size() / 2);
    if (cand.size() > cand_.size()) cand_ = DeviceArray<double>(cand.size() * 2);
    if (M) cand_.upload(cand.data(), cand.size(), a1_.stream());
    check(mkf_pdaf_associate(a1_.handle(), a2_.handle(), frame, roi, M ? cand_.data() : nullptr, M, Pa_,
                             clutter_, meas1_.data(), meas2_.data(), nullptr, nullptr, a1_.stream()),
          "mkf_pdaf_associate");
    unsigned mask1 = (1u << a1_.m) - 1u, mask2 = (1u << a2_.m) - 1u;
    if (M == 0) { mask1 &= ~0xCu; mask2 &= ~0xCu; }   // no candidate: hand rows unused
    a1_.update(meas1_.data(), mask1, frame);
    a2_.update(meas2_.data(), mask2, frame);
    return true;
  }

 private:
  RaoParticleFilter& a1_;
  RaoParticleFilter& a2_;
  double Pa_, clutter_;
  DeviceArray<double> meas1_, meas2_, cand_;
  DeviceArray<uint8_t> blur_;
  bool init_ = false;
};

// ------------------------------------- decode, get3Dpose and publish2Dpos record
class PoseDecoder {
 public:
  PoseDecoder(const std::vector<double>& Hpca, const std::vector<double>& mpca, int d, const double Kc[9],
              cudaStream_t stream = nullptr)
      : d(d), F(static_cast<int>(mpca.size())), H_(Hpca), m_(mpca), status_(1), stream_(stream) {
    for (int q = 0; q < 9; ++q) Kc_[q] = Kc[q];
    int z = 0;
    status_.upload(&z, 1, stream_);
  }
  // B estimates (B*d, device) -> e (B*F) and 3-D points (B*15, or nullptr)
  void decode(const double* d_x, int B, double* d_e, double* d_pos3d) {
    check(mkf_pose_decode(d_x, B, d, F, H_.data(), m_.data(), Kc_, d_e, d_pos3d, status_.data(), stream_),
          "mkf_pose_decode");
  }
  const int d, F;

 private:
  DeviceArray<double> H_, m_;
  DeviceArray<int> status_;
  double Kc_[9];
  cudaStream_t stream_;
};

// ---------------------------------------- batched bootstrap PFs, one launch
// Independent bootstrap trackers (the pf2D structure, pf2D.cpp:148-210, with
// the mixture motion model of my_gmm) of uneven length, particle count and
// clutter, all run by one persistent kernel.  Track b's frames are the global
// frames [frame_base, frame_base + n_frames); detections are per (global frame,
// joint) lists, det_off (n_frames_total * J + 1 offsets) into det (x, y pairs).
class BatchedBootstrapPF {
 public:
  BatchedBootstrapPF(const mkf_bpf_models& models, const std::vector<mkf_bpf_track>& tracks, int64_t n_frames_total)
      : d(models.d), J(models.J), n_tracks(static_cast<int>(tracks.size())), n_frames_total(n_frames_total) {
    check(mkf_bpf_batch_create(&models, n_tracks, tracks.data(), n_frames_total, &h_), "mkf_bpf_batch_create");
  }
  ~BatchedBootstrapPF() { if (h_) mkf_bpf_batch_destroy(h_); }
  BatchedBootstrapPF(const BatchedBootstrapPF&) = delete;
  BatchedBootstrapPF& operator=(const BatchedBootstrapPF&) = delete;
  // launch shape and code variant (MKF_BPF_*); the defaults are the fastest measured
  void setTuning(int block_threads, int ctas_per_sm) {
    check(mkf_bpf_batch_set_tuning(h_, block_threads, ctas_per_sm), "mkf_bpf_batch_set_tuning");
  }
  void setVariant(int flags) { check(mkf_bpf_batch_set_variant(h_, flags), "mkf_bpf_batch_set_variant"); }
  // device buffers: est (n_frames_total * d), loglik and ess (n_frames_total),
  // status (n_tracks); asynchronous on the stream
  void run(const int* d_det_off, const float* d_det, float* d_est, float* d_loglik, float* d_ess, int* d_status,
           cudaStream_t stream = nullptr) {
    check(mkf_bpf_batch_run(h_, d_det_off, d_det, d_est, d_loglik, d_ess, d_status, stream), "mkf_bpf_batch_run");
  }
  // host buffers (copied in and out, synchronous); outputs are resized
  void run(const std::vector<int>& det_off, const std::vector<float>& det, std::vector<float>& est,
           std::vector<float>& loglik, std::vector<float>& ess, std::vector<int>& status,
           cudaStream_t stream = nullptr) {
    const size_t G = static_cast<size_t>(n_frames_total);
    if (det_off.size() != G * J + 1 || det.size() % 2)
      throw Error(MKF_ERR_ARG, "BatchedBootstrapPF::run: det_off needs n_frames_total * J + 1 entries, det pairs");
    est.resize(G * d); loglik.resize(G); ess.resize(G); status.resize(static_cast<size_t>(n_tracks));
    static const float no_det[2] = {0.0f, 0.0f};
    check(mkf_bpf_batch_run_host(h_, det_off.data(), det.empty() ? no_det : det.data(),
                                 static_cast<int64_t>(det.size() / 2), est.data(),
                                 loglik.data(), ess.data(), status.data(), stream),
          "mkf_bpf_batch_run_host");
  }
  int lastGrid() const {
    int g = 0;
    check(mkf_bpf_batch_last_grid(h_, &g), "mkf_bpf_batch_last_grid");
    return g;
  }
  const int d, J, n_tracks;
  const int64_t n_frames_total;

 private:
  mkf_bpf_batch_t h_ = nullptr;
};

}  // namespace mkf
