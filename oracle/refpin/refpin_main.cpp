// refpin_main.cpp -- runs the reference's own filter classes (KF_model,
// my_gmm, ParticleFilter from KF_model.cpp, my_gmm.cpp and pf2DRao.cpp,
// compiled unmodified from the reference checkout against the stand-in headers
// in shim/) on the cases read from stdin, and prints what they compute.
// TEST INFRASTRUCTURE ONLY: tests/golden/make_refpin_golden.py runs it to make
// the golden vectors that pin the oracle.
//
// Input: whitespace-separated tokens.  Each case starts with a keyword:
//   CONV c                  Cholesky diagonal convention of the stand-in (24 or 3)
//   KF d m F B Q H BH R x P z
//                           KF_model::predict then ::update (KF_model.cpp:11-25)
//   LOADG K d Fd {u s w g}*K Hpca mpca
//                           my_gmm::loadGaussian per component (my_gmm.cpp:45-75)
//   RESAMPLE L N w u i0 {f}*N
//                           ParticleFilter::resample (pf2DRao.cpp:175-210) with the
//                           injected uniform u, first integer draw i0 and the N
//                           integers of its all-zero branch
//   MVN m x u S             ParticleFilter::chol and ::mvnpdf (pf2DRao.cpp:34-67)
//   RBPF K d Fd N T {u s w g}*K Hpca mpca bins {z u_ind u_anc {f}*N}*T
//                           loadGaussian, resetTracker(bins), then T times
//                           ParticleFilter::update(z) (pf2DRao.cpp:125-158) with
//                           injected uniforms (f: the integers of the second
//                           resample's all-zero branch), printing the tracks and
//                           getEstimator (pf2DRao.cpp:23-31) after each
// Matrices are given row-major with their sizes implied by the case.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "pf2DRao.h"

namespace cv {
static int g_conv = 24;
int cholesky_convention() { return g_conv; }
std::deque<double>& injected_uniforms() {
  static std::deque<double> q;
  return q;
}
std::deque<int>& injected_ints() {
  static std::deque<int> q;
  return q;
}
std::deque<double>& injected_normals() {
  static std::deque<double> q;
  return q;
}
}  // namespace cv

// the protected Gaussian pieces of ParticleFilter, reached from a subclass
class PinFilter : public ParticleFilter {
 public:
  explicit PinFilter(int n) : ParticleFilter(n) {}
  double density(cv::Mat x, cv::Mat u, cv::Mat s) { return mvnpdf(x, u, s); }
  cv::Mat factor(cv::Mat s) { return chol(s); }
};

static cv::Mat read_mat(int r, int c) {
  cv::Mat m = cv::Mat::zeros(r, c, CV_64F);
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j) std::cin >> m.at<double>(i, j);
  return m;
}

static void print_mat(const char* tag, const cv::Mat& m) {
  std::printf("%s %d %d", tag, m.rows, m.cols);
  for (int i = 0; i < m.rows; ++i)
    for (int j = 0; j < m.cols; ++j) std::printf(" %.17g", m.at<double>(i, j));
  std::printf("\n");
}

static void load_components(ParticleFilter& pf, int K, int d, int Fd) {
  std::vector<cv::Mat> u(K), s(K);
  std::vector<double> w(K), g(K);
  for (int k = 0; k < K; ++k) {
    u[k] = read_mat(1, d);
    s[k] = read_mat(d, d);
    std::cin >> w[k] >> g[k];
  }
  cv::Mat H = read_mat(d, Fd), m = read_mat(1, Fd);
  for (int k = 0; k < K; ++k) pf.gmm.loadGaussian(u[k], s[k], H, m, w[k], g[k]);
}

int main() {
  std::string cmd;
  while (std::cin >> cmd) {
    if (cmd == "CONV") {
      std::cin >> cv::g_conv;
    } else if (cmd == "KF") {
      int d, m;
      std::cin >> d >> m;
      KF_model kf;
      kf.F = read_mat(d, d);
      kf.B = read_mat(d, 1);
      kf.Q = read_mat(d, d);
      kf.H = read_mat(m, d);
      kf.BH = read_mat(m, 1);
      kf.R = read_mat(m, m);
      cv::Mat x = read_mat(d, 1), P = read_mat(d, d), z = read_mat(m, 1);
      kf.predict(x, P);
      print_mat("xp", x);
      print_mat("Pp", P);
      kf.update(z, x, P);
      print_mat("xu", x);
      print_mat("Pu", P);
    } else if (cmd == "LOADG") {
      int K, d, Fd;
      std::cin >> K >> d >> Fd;
      ParticleFilter pf(1);
      load_components(pf, K, d, Fd);
      for (int k = 0; k < K; ++k) {
        const KF_model& t = pf.gmm.KFtracker[k];
        print_mat("F", t.F);
        print_mat("B", t.B);
        print_mat("Q", t.Q);
        print_mat("H", t.H);
        print_mat("BH", t.BH);
        print_mat("R", t.R);
      }
    } else if (cmd == "RESAMPLE") {
      int L, N;
      std::cin >> L >> N;
      std::vector<double> w(L);
      for (double& v : w) std::cin >> v;
      double u;
      int i0;
      std::cin >> u >> i0;
      cv::injected_uniforms().push_back(u);
      cv::injected_ints().push_back(i0);
      for (int i = 0; i < N; ++i) {
        int f;
        std::cin >> f;
        cv::injected_ints().push_back(f);
      }
      ParticleFilter pf(N);
      std::vector<int> idx = pf.resample(w, N);
      std::printf("idx %d", (int)idx.size());
      for (int v : idx) std::printf(" %d", v);
      std::printf("\n");
      cv::injected_uniforms().clear();
      cv::injected_ints().clear();
    } else if (cmd == "MVN") {
      int m;
      std::cin >> m;
      cv::Mat x = read_mat(m, 1), u = read_mat(m, 1), S = read_mat(m, m);
      PinFilter pf(1);
      print_mat("chol", pf.factor(S));
      std::printf("p %.17g\n", pf.density(x, u, S));
    } else if (cmd == "RBPF") {
      int K, d, Fd, N, T;
      std::cin >> K >> d >> Fd >> N >> T;
      ParticleFilter pf(N);
      load_components(pf, K, d, Fd);
      std::vector<int> bins(N);
      for (int& b : bins) std::cin >> b;
      pf.gmm.resetTracker(bins);
      for (int t = 0; t < T; ++t) {
        cv::Mat z = read_mat(6, N);
        double ui, ua;
        std::cin >> ui >> ua;
        // each resample call first draws an integer (pf2DRao.cpp:180), then its
        // uniform, or N integers in its all-zero branch (only the second call's
        // weights can all be zero)
        cv::injected_ints().push_back(0);
        cv::injected_ints().push_back(0);
        for (int j = 0; j < N; ++j) {
          int f;
          std::cin >> f;
          cv::injected_ints().push_back(f);
        }
        cv::injected_uniforms().push_back(ui);
        cv::injected_uniforms().push_back(ua);
        pf.update(z);
        std::printf("frame %d %d\n", t, (int)cv::injected_ints().size() == 0 ? 1 : 0);
        for (int j = 0; j < N; ++j) {
          print_mat("x", pf.gmm.tracks[j].state);
          print_mat("P", pf.gmm.tracks[j].cov);
        }
        print_mat("est", pf.getEstimator());
        cv::injected_uniforms().clear();
        cv::injected_ints().clear();
      }
    } else {
      std::fprintf(stderr, "unknown case %s\n", cmd.c_str());
      return 2;
    }
  }
  return 0;
}
