// mkf_harness -- standalone, ROS-free replacement of the reference's PFTracker
// node (pfPose.cpp, pfPoseTracker.cpp) over libmkf_gb300.so.
//
//   mkf_harness track --arm1 L.yml --arm2 R.yml --frames in.bin --out out.bin
//                     [--particles 500] [--seed S] [--pa 0.05] [--clutter 1e-4]
//                     [--own-gamma]
//     Loads both arm models as the PFTracker constructor does (pfPose.cpp:24-71:
//     means, covs, weights, pca_proj, pca_mean; gamma of BOTH arms from the
//     right-arm file unless --own-gamma), resets the trackers, then runs the
//     frame loop of PFTracker::callback (pfPose.cpp:332-385) over the frame
//     records of in.bin: PDAF association of the hand candidates and both arm
//     updates when the frame has a face ROI, a skipped frame otherwise.  After
//     the loop the estimates of all frames are decoded on the device in one
//     batch (e = H_pca^T x + m_pca, get3Dpose, the publish2Dpos points) and
//     written to out.bin.  Prints one JSON line with the frame rate.
//
//   mkf_harness yaml-roundtrip in.yml out.yml
//     Reads an OpenCV-YAML file and writes it back (model-file I/O check).
//
// Frame file (little-endian): "MKFFRM01", int32 n_frames, then per frame:
//   int32 frame_id, int32 has_roi, double roi[8] (x_offset, y_offset, width,
//   height per arm), int32 M, double cand[2M] (hand candidate x, y).
// Version "MKFFRM02" adds int32 width, height after n_frames and a MONO8
// likelihood image (height x width bytes) after each frame's candidates; the
// harness then runs the reference's image path (blur, 10 N proposals per arm,
// likelihood weights) instead of the candidate list.
// Output file: "MKFOUT01", int32 n_frames, int32 d, int32 F, then per frame:
//   int32 frame_id, int32 valid, double est[2][d], double e[2][F],
//   double points[8][2] (hand1, hand2, head, neck, elbow1, elbow2, shoulder1,
//   shoulder2), double pos3d[2][3][5].
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mkf_gb300.hpp"
#include "mkf_yaml.hpp"

namespace {

struct Frame {
  int32_t id = 0, has_roi = 0;
  double roi[8] = {0};
  std::vector<double> cand;
  std::vector<uint8_t> like;   // MONO8 likelihood image (frame files of version 2)
};

struct FrameFile {
  std::vector<Frame> frames;
  int width = 0, height = 0;   // likelihood image size (0: detection-list frames)
};

template <class T>
void rd(std::ifstream& f, T* v, size_t n = 1) {
  f.read(reinterpret_cast<char*>(v), static_cast<std::streamsize>(sizeof(T) * n));
  if (!f) throw std::runtime_error("frame file truncated");
}
template <class T>
void wr(std::ofstream& f, const T* v, size_t n = 1) {
  f.write(reinterpret_cast<const char*>(v), static_cast<std::streamsize>(sizeof(T) * n));
}

FrameFile read_frames(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  char magic[8];
  rd(f, magic, 8);
  const bool v2 = std::memcmp(magic, "MKFFRM02", 8) == 0;
  if (!v2 && std::memcmp(magic, "MKFFRM01", 8) != 0) throw std::runtime_error("not a frame file: " + path);
  FrameFile ff;
  int32_t n = 0;
  rd(f, &n);
  if (n < 0) throw std::runtime_error("bad frame count");
  if (v2) {
    int32_t wh[2];
    rd(f, wh, 2);
    if (wh[0] < 8 || wh[1] < 8 || wh[0] > 8192 || wh[1] > 8192) throw std::runtime_error("bad image size");
    ff.width = wh[0];
    ff.height = wh[1];
  }
  ff.frames.resize(static_cast<size_t>(n));
  for (Frame& fr : ff.frames) {
    rd(f, &fr.id);
    rd(f, &fr.has_roi);
    rd(f, fr.roi, 8);
    int32_t M = 0;
    rd(f, &M);
    if (M < 0 || M > 65536) throw std::runtime_error("bad candidate count");
    fr.cand.resize(static_cast<size_t>(2 * M));
    if (M) rd(f, fr.cand.data(), fr.cand.size());
    if (v2) {
      fr.like.resize(static_cast<size_t>(ff.width) * ff.height);
      rd(f, fr.like.data(), fr.like.size());
    }
  }
  return ff;
}

struct ArmModel {
  mkf::yaml::Matrix means, covs, weights, pca_proj, pca_mean, gamma;
};

ArmModel load_arm(const mkf::yaml::Document& doc) {
  ArmModel a;
  a.means = doc.matrix("means");
  a.covs = doc.matrix("covs");
  a.weights = doc.matrix("weights");
  a.pca_proj = doc.matrix("pca_proj");
  a.pca_mean = doc.matrix("pca_mean");
  a.gamma = doc.matrix("gamma");
  return a;
}

// PFTracker constructor body for one arm (pfPose.cpp:58-71)
void load_filter(mkf::RaoParticleFilter& pf, const ArmModel& a, const mkf::yaml::Matrix& gamma) {
  const int K = a.means.rows, d = a.means.cols, F = a.pca_proj.cols;
  if (K != pf.K || d != pf.d) throw std::runtime_error("model size differs from the filter's");
  if (a.covs.rows != K * d || a.covs.cols != d || a.pca_proj.rows != d || a.pca_mean.rows * a.pca_mean.cols != F ||
      static_cast<int>(a.weights.data.size()) < K || static_cast<int>(gamma.data.size()) < K)
    throw std::runtime_error("model matrices have inconsistent sizes");
  for (int k = 0; k < K; ++k) {
    std::vector<double> u(a.means.data.begin() + static_cast<size_t>(k) * d,
                          a.means.data.begin() + static_cast<size_t>(k + 1) * d);
    std::vector<double> s(a.covs.data.begin() + static_cast<size_t>(k) * d * d,
                          a.covs.data.begin() + static_cast<size_t>(k + 1) * d * d);
    // weights1.at<double>(0, k), g.at<double>(0, k) on a K x 1 matrix = element k
    pf.gmm.loadGaussian(k, u, s, a.pca_proj.data, a.pca_mean.data, a.weights.data[k], gamma.data[k]);
  }
  std::vector<double> Hd(static_cast<size_t>(2) * d), hb(2);
  for (int r = 0; r < d; ++r) {
    Hd[r] = a.pca_proj.at(r, 0);
    Hd[d + r] = a.pca_proj.at(r, 1);
  }
  hb[0] = a.pca_mean.data[0];
  hb[1] = a.pca_mean.data[1];
  pf.setHandDecode(Hd, hb);
  pf.gmm.resetTracker();
}

int cmd_track(int argc, char** argv) {
  std::string arm1, arm2, frames_path, out_path;
  mkf::TrackerConfig cfg;
  int& N = cfg.particles;
  uint64_t& seed = cfg.seed;
  double &Pa = cfg.Pa, &clutter = cfg.clutter;
  bool own_gamma = false;
  for (int i = 2; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw std::runtime_error("missing value for " + a);
      return argv[++i];
    };
    if (a == "--arm1") arm1 = next();
    else if (a == "--arm2") arm2 = next();
    else if (a == "--frames") frames_path = next();
    else if (a == "--out") out_path = next();
    else if (a == "--particles") N = std::stoi(next());
    else if (a == "--seed") seed = std::stoull(next());
    else if (a == "--pa") Pa = std::stod(next());
    else if (a == "--clutter") clutter = std::stod(next());
    else if (a == "--own-gamma") own_gamma = true;
    else throw std::runtime_error("unknown option " + a);
  }
  if (arm1.empty() || arm2.empty() || frames_path.empty() || out_path.empty())
    throw std::runtime_error("track needs --arm1 --arm2 --frames --out");
  const ArmModel m1 = load_arm(mkf::yaml::load(arm1)), m2 = load_arm(mkf::yaml::load(arm2));
  const FrameFile ff = read_frames(frames_path);
  const std::vector<Frame>& frames = ff.frames;
  const bool image_mode = ff.width > 0;
  const int K = m1.means.rows, d = m1.means.cols, F = m1.pca_proj.cols;
  const int T = static_cast<int>(frames.size());

  cudaStream_t s = nullptr;
  mkf::cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
  {
    mkf::RaoParticleFilter pf1(N, d, 6, K, MKF_MEAS_LINEAR, seed, 0, s), pf2(N, d, 6, K, MKF_MEAS_LINEAR, seed, 1, s);
    load_filter(pf1, m1, own_gamma ? m1.gamma : m2.gamma);    // fs2["gamma"] for both (pfPose.cpp:52-53)
    load_filter(pf2, m2, m2.gamma);
    mkf::PoseTracker tracker(pf1, pf2, Pa, clutter);
    mkf::DeviceArray<double> est1(static_cast<size_t>(T) * d + 1), est2(static_cast<size_t>(T) * d + 1);
    // likelihood images are staged into a ring of device buffers up front (the
    // image transport is the caller's, as the ROS topics were)
    std::vector<mkf::DeviceArray<uint8_t>> like;
    if (image_mode)
      for (const Frame& fr : frames) like.emplace_back(fr.like);
    std::vector<int> valid(static_cast<size_t>(T), 0);
    mkf::cuda_check(cudaStreamSynchronize(s), "sync");
    cudaEvent_t e0, e1;
    mkf::cuda_check(cudaEventCreate(&e0), "event");
    mkf::cuda_check(cudaEventCreate(&e1), "event");
    const auto w0 = std::chrono::steady_clock::now();
    mkf::cuda_check(cudaEventRecord(e0, s), "event");
    for (int t = 0; t < T; ++t) {
      const Frame& fr = frames[t];
      const bool ok = image_mode
                          ? tracker.stepImage(static_cast<uint32_t>(fr.id), fr.has_roi ? fr.roi : nullptr,
                                              like[t].data(), ff.width, ff.height, ff.width,
                                              cfg.candidates_per_particle * N)
                          : tracker.step(static_cast<uint32_t>(fr.id), fr.has_roi ? fr.roi : nullptr, fr.cand);
      if (ok) {
        pf1.estimateInto(est1.data() + static_cast<size_t>(t) * d);
        pf2.estimateInto(est2.data() + static_cast<size_t>(t) * d);
        valid[t] = 1;
      }
    }
    // batched decode of every frame's estimate (skipped frames decode zeros and are flagged invalid)
    mkf::PoseDecoder dec1(m1.pca_proj.data, m1.pca_mean.data, d, cfg.K, s),
        dec2(m2.pca_proj.data, m2.pca_mean.data, d, cfg.K, s);
    mkf::DeviceArray<double> e_1(static_cast<size_t>(T) * F + 1), e_2(static_cast<size_t>(T) * F + 1);
    mkf::DeviceArray<double> p3_1(static_cast<size_t>(T) * 15 + 1), p3_2(static_cast<size_t>(T) * 15 + 1);
    mkf::DeviceArray<double> pts(static_cast<size_t>(T) * 16 + 1);
    dec1.decode(est1.data(), T, e_1.data(), p3_1.data());
    dec2.decode(est2.data(), T, e_2.data(), p3_2.data());
    mkf::check(mkf_pose2d_record(e_1.data(), e_2.data(), T, F, pts.data(), s), "mkf_pose2d_record");
    std::vector<double> h_est1 = est1.to_host(s), h_est2 = est2.to_host(s), h_e1 = e_1.to_host(s),
                        h_e2 = e_2.to_host(s), h_p1 = p3_1.to_host(s), h_p2 = p3_2.to_host(s), h_pts = pts.to_host(s);
    mkf::cuda_check(cudaEventRecord(e1, s), "event");
    mkf::cuda_check(cudaEventSynchronize(e1), "event");
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    float ms = 0.0f;
    mkf::cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);

    std::ofstream f(out_path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + out_path);
    f.write("MKFOUT01", 8);
    const int32_t hdr[3] = {T, d, F};
    wr(f, hdr, 3);
    for (int t = 0; t < T; ++t) {
      const int32_t rec[2] = {frames[t].id, valid[t]};
      wr(f, rec, 2);
      wr(f, &h_est1[static_cast<size_t>(t) * d], d);
      wr(f, &h_est2[static_cast<size_t>(t) * d], d);
      wr(f, &h_e1[static_cast<size_t>(t) * F], F);
      wr(f, &h_e2[static_cast<size_t>(t) * F], F);
      wr(f, &h_pts[static_cast<size_t>(t) * 16], 16);
      wr(f, &h_p1[static_cast<size_t>(t) * 15], 15);
      wr(f, &h_p2[static_cast<size_t>(t) * 15], 15);
    }
    int nvalid = 0;
    for (int v : valid) nvalid += v;
    std::printf("{\"harness\": \"track\", \"input\": \"%s\", \"frames\": %d, \"valid_frames\": %d, \"particles_per_arm\": %d, "
                "\"wall_s\": %.6f, \"device_s\": %.6f, \"frames_per_s\": %.3f, \"arm_frames_per_s\": %.3f, "
                "\"status\": [%d, %d]}\n",
                image_mode ? "likelihood images" : "candidate lists", T, nvalid, N, wall, ms / 1000.0, T / wall, 2.0 * nvalid / wall, pf1.status(), pf2.status());
  }
  cudaStreamDestroy(s);
  return 0;
}

int cmd_yaml_roundtrip(int argc, char** argv) {
  if (argc != 4) throw std::runtime_error("yaml-roundtrip needs <in.yml> <out.yml>");
  mkf::yaml::save(argv[3], mkf::yaml::load(argv[2]));
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: mkf_harness track ... | yaml-roundtrip in.yml out.yml\n");
    return 2;
  }
  try {
    const std::string cmd = argv[1];
    if (cmd == "track") return cmd_track(argc, argv);
    if (cmd == "yaml-roundtrip") return cmd_yaml_roundtrip(argc, argv);
    std::fprintf(stderr, "unknown command %s\n", cmd.c_str());
    return 2;
  } catch (const mkf::Error& e) {
    std::fprintf(stderr, "mkf error %d: %s\n", e.status, e.what());
    return 1;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
}
