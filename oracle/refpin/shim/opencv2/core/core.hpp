// Stand-in for the few OpenCV core pieces that the reference's filter sources
// (KF_model.cpp, my_gmm.cpp, pf2DRao.cpp) use, so that those files compile
// unmodified from the reference checkout for the oracle pin (oracle/refpin).
// TEST INFRASTRUCTURE ONLY.  This is not OpenCV: it restates the documented
// behaviour of the calls the reference makes, for CV_64F (and the two-channel
// CV_64FC2 of getSamples), in this project's own code:
//  * Mat is a reference-counted header; copy and copy-assign share the data
//    (shallow), clone() copies it; row/col/diag/rowRange/operator()(Range,Range)
//    are views that share the data.
//  * Arithmetic (A*B, A+B, A-B, s*A, A-s, A.t(), A.inv(), Mat::eye/zeros)
//    yields a MatExpr.  Assigning a MatExpr to a Mat that already has the
//    result's size and type writes into that Mat's existing data (so every Mat
//    sharing it sees the new values); otherwise the Mat is re-bound to the new
//    data.  That is the rule behind the reference's shared-buffer effect after
//    its copy-assign resampling (pf2DRao.cpp:153-156 with KF_model.cpp:13-24).
//    A sum with an empty operand is the other operand.
//  * inv(): Gauss-Jordan elimination with partial pivoting (the LU default).
//  * Cholesky(A, astep, m, 0, 0, 0): in-place lower factor; the diagonal keeps
//    1 / L_ii (cholesky_convention() == 24) or L_ii (== 3), the two behaviours
//    of the call across OpenCV versions that the reference's chol() reads.
//  * RNG / randn draw from queues the driver fills (injected draws).
#ifndef MKF_REFPIN_CORE_HPP
#define MKF_REFPIN_CORE_HPP

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <deque>
#include <memory>
#include <stdexcept>
#include <vector>

#define CV_64F 6
#define CV_64FC2 14
#define CV_REDUCE_SUM 0

namespace cv {

struct Range {
  int start, end;
  Range(int s, int e) : start(s), end(e) {}
  static Range all() { return Range(0, -1); }
};

struct Scalar {
  double v[4];
  Scalar(double a = 0, double b = 0, double c = 0, double d = 0) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
  static Scalar all(double a) { return Scalar(a, a, a, a); }
  double operator[](int i) const { return v[i]; }
  double& operator[](int i) { return v[i]; }
};

class MatExpr;

class Mat {
 public:
  int rows, cols;
  size_t step;                       // bytes between rows
  std::shared_ptr<std::vector<double>> buf;
  double* data_;                     // first element of this header's view
  int cn;                            // channels (1, or 2 for CV_64FC2)

  Mat() : rows(0), cols(0), step(0), data_(nullptr), cn(1) {}
  Mat(int r, int c, int type) { alloc(r, c, type == CV_64FC2 ? 2 : 1); }
  Mat(const Mat& m) = default;
  Mat(const MatExpr& e);
  Mat& operator=(const Mat& m) = default;
  Mat& operator=(const MatExpr& e);
  // a view: rows [r0, r1), cols [c0, c1)
  Mat operator()(const Range& rr, const Range& cr) const {
    const int r1 = rr.end < 0 ? rows : rr.end, c1 = cr.end < 0 ? cols : cr.end;
    Mat v = *this;
    v.rows = r1 - rr.start;
    v.cols = c1 - cr.start;
    v.data_ = data_ + (size_t)rr.start * ld() + (size_t)cr.start * cn;
    return v;
  }

  bool empty() const { return data_ == nullptr || rows == 0 || cols == 0; }
  int type() const { return cn == 2 ? CV_64FC2 : CV_64F; }
  int channels() const { return cn; }
  size_t ld() const { return step / sizeof(double); }     // row stride in doubles
  template <typename T> T* ptr(int r = 0) { return reinterpret_cast<T*>(data_ + (size_t)r * ld()); }
  template <typename T> const T* ptr(int r = 0) const { return reinterpret_cast<const T*>(data_ + (size_t)r * ld()); }
  template <typename T> T& at(int r, int c) { return *reinterpret_cast<T*>(data_ + (size_t)r * ld() + (size_t)c * cn); }
  template <typename T> const T& at(int r, int c) const {
    return *reinterpret_cast<const T*>(data_ + (size_t)r * ld() + (size_t)c * cn);
  }
  // one index: element i of a row or column vector
  template <typename T> T& at(int i) { return rows == 1 ? at<T>(0, i) : at<T>(i, 0); }
  template <typename T> const T& at(int i) const { return rows == 1 ? at<T>(0, i) : at<T>(i, 0); }

  Mat row(int r) const { return (*this)(Range(r, r + 1), Range(0, cols)); }
  Mat col(int c) const { return (*this)(Range(0, rows), Range(c, c + 1)); }
  Mat rowRange(const Range& r) const { return (*this)(r, Range(0, cols)); }
  Mat colRange(const Range& c) const { return (*this)(Range(0, rows), c); }
  // diagonal d (d > 0 above, d < 0 below) as a column vector view
  Mat diag(int d = 0) const {
    Mat v = *this;
    const int r0 = d < 0 ? -d : 0, c0 = d > 0 ? d : 0;
    const int n = std::min(rows - r0, cols - c0);
    v.rows = n > 0 ? n : 0;
    v.cols = 1;
    v.data_ = data_ + (size_t)r0 * ld() + c0;
    v.step = step + sizeof(double);
    return v;
  }
  Mat clone() const {
    Mat m(rows, cols, type());
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols * cn; ++c) m.data_[(size_t)r * m.ld() + c] = data_[(size_t)r * ld() + c];
    return m;
  }
  void copyTo(Mat dst) const;                     // into dst's data (a view of the same size)
  void copyTo(std::vector<double>& v) const {
    v.resize((size_t)rows * cols);
    size_t k = 0;
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c) v[k++] = at<double>(r, c);
  }
  void convertTo(Mat& dst, int) const { dst = clone(); }
  Mat& operator*=(double s) {
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols * cn; ++c) data_[(size_t)r * ld() + c] *= s;
    return *this;
  }
  MatExpr t() const;
  MatExpr inv() const;
  static MatExpr zeros(int r, int c, int type);
  static MatExpr eye(int r, int c, int type);

  void alloc(int r, int c, int ch) {
    rows = r; cols = c; cn = ch;
    buf = std::make_shared<std::vector<double>>((size_t)r * c * ch, 0.0);
    data_ = buf->data();
    step = (size_t)c * ch * sizeof(double);
  }
};

// an evaluated expression (the result is computed eagerly; only the
// assignment rule differs from a Mat)
class MatExpr {
 public:
  Mat m;
  explicit MatExpr(const Mat& r) : m(r) {}
  operator Mat() const { return m; }
  MatExpr t() const { return m.t(); }
  MatExpr inv() const { return m.inv(); }
  Mat col(int c) const { return m.col(c); }
  Mat row(int r) const { return m.row(r); }
};

inline Mat::Mat(const MatExpr& e) : Mat(e.m) {}

inline void copy_values(const Mat& src, Mat& dst) {
  for (int r = 0; r < src.rows; ++r)
    for (int c = 0; c < src.cols * src.cn; ++c)
      dst.data_[(size_t)r * dst.ld() + c] = src.data_[(size_t)r * src.ld() + c];
}

inline Mat& Mat::operator=(const MatExpr& e) {
  if (!empty() && rows == e.m.rows && cols == e.m.cols && cn == e.m.cn) {
    if (data_ != e.m.data_) {
      const Mat tmp = e.m.clone();      // the expression may read this Mat's own data
      copy_values(tmp, *this);
    }
  } else {
    *this = e.m;
  }
  return *this;
}

inline void Mat::copyTo(Mat dst) const {
  if (!dst.empty() && dst.rows == rows && dst.cols == cols && dst.cn == cn) copy_values(*this, dst);
  else throw std::runtime_error("refpin shim: copyTo a view of another size");
}

inline MatExpr Mat::t() const {
  Mat r(cols, rows, CV_64F);
  for (int i = 0; i < rows; ++i)
    for (int j = 0; j < cols; ++j) r.at<double>(j, i) = at<double>(i, j);
  return MatExpr(r);
}

inline MatExpr Mat::inv() const {
  const int n = rows;
  if (n != cols) throw std::runtime_error("refpin shim: inv of a non-square matrix");
  std::vector<double> a((size_t)n * 2 * n);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < 2 * n; ++c) a[(size_t)r * 2 * n + c] = c < n ? at<double>(r, c) : (c - n == r ? 1.0 : 0.0);
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[(size_t)r * 2 * n + c]) > std::fabs(a[(size_t)p * 2 * n + c])) p = r;
    if (p != c)
      for (int k = 0; k < 2 * n; ++k) std::swap(a[(size_t)c * 2 * n + k], a[(size_t)p * 2 * n + k]);
    const double d = a[(size_t)c * 2 * n + c];
    if (d == 0.0) return MatExpr(Mat(n, n, CV_64F));   // singular: zeros, as the LU inverse reports
    for (int k = 0; k < 2 * n; ++k) a[(size_t)c * 2 * n + k] /= d;
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[(size_t)r * 2 * n + c];
      if (f != 0.0)
        for (int k = 0; k < 2 * n; ++k) a[(size_t)r * 2 * n + k] -= f * a[(size_t)c * 2 * n + k];
    }
  }
  Mat r(n, n, CV_64F);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) r.at<double>(i, j) = a[(size_t)i * 2 * n + n + j];
  return MatExpr(r);
}

inline MatExpr Mat::zeros(int r, int c, int type) { return MatExpr(Mat(r, c, type)); }
inline MatExpr Mat::eye(int r, int c, int type) {
  Mat m(r, c, type);
  for (int i = 0; i < std::min(r, c); ++i) m.at<double>(i, i) = 1.0;
  return MatExpr(m);
}

inline MatExpr operator*(const Mat& a, const Mat& b) {
  if (a.cols != b.rows) throw std::runtime_error("refpin shim: matrix product of mismatched sizes");
  Mat r(a.rows, b.cols, CV_64F);
  for (int i = 0; i < a.rows; ++i)
    for (int j = 0; j < b.cols; ++j) {
      double s = 0.0;
      for (int k = 0; k < a.cols; ++k) s += a.at<double>(i, k) * b.at<double>(k, j);
      r.at<double>(i, j) = s;
    }
  return MatExpr(r);
}
inline MatExpr operator*(double s, const Mat& a) {
  Mat r = a.clone();
  r *= s;
  return MatExpr(r);
}
inline MatExpr operator*(const Mat& a, double s) { return s * a; }
inline MatExpr elementwise(const Mat& a, const Mat& b, double sb) {
  if (a.empty()) return sb * b;                // an empty operand is absent
  if (b.empty()) return MatExpr(a.clone());
  if (a.rows != b.rows || a.cols != b.cols) throw std::runtime_error("refpin shim: sum of mismatched sizes");
  Mat r = a.clone();
  for (int i = 0; i < a.rows; ++i)
    for (int j = 0; j < a.cols * a.cn; ++j) r.data_[(size_t)i * r.ld() + j] += sb * b.data_[(size_t)i * b.ld() + j];
  return MatExpr(r);
}
inline MatExpr operator+(const Mat& a, const Mat& b) { return elementwise(a, b, 1.0); }
inline MatExpr operator-(const Mat& a, const Mat& b) { return elementwise(a, b, -1.0); }
inline MatExpr operator-(const Mat& a, double s) {
  Mat r = a.clone();
  for (int i = 0; i < r.rows; ++i)
    for (int j = 0; j < r.cols; ++j) r.at<double>(i, j) -= s;
  return MatExpr(r);
}
inline MatExpr operator+(const Mat& a, double s) { return a - (-s); }
// MatExpr operands go through the Mat conversion; these keep the overloads unambiguous
inline MatExpr operator*(const MatExpr& a, const MatExpr& b) { return a.m * b.m; }
inline MatExpr operator*(const MatExpr& a, const Mat& b) { return a.m * b; }
inline MatExpr operator*(const Mat& a, const MatExpr& b) { return a * b.m; }
inline MatExpr operator*(double s, const MatExpr& a) { return s * a.m; }
inline MatExpr operator+(const MatExpr& a, const MatExpr& b) { return a.m + b.m; }
inline MatExpr operator+(const MatExpr& a, const Mat& b) { return a.m + b; }
inline MatExpr operator+(const Mat& a, const MatExpr& b) { return a + b.m; }
inline MatExpr operator-(const MatExpr& a, const MatExpr& b) { return a.m - b.m; }
inline MatExpr operator-(const MatExpr& a, const Mat& b) { return a.m - b; }
inline MatExpr operator-(const Mat& a, const MatExpr& b) { return a - b.m; }
inline MatExpr operator-(const MatExpr& a, double s) { return a.m - s; }

// -------------------------------------------------------------- free functions
int cholesky_convention();                         // 24 or 3 (set by the driver)

// In-place Cholesky of the m x m matrix A (row step astep bytes): the lower
// factor L below the diagonal; on the diagonal 1 / L_ii (convention 24) or L_ii
// (convention 3).  Returns false if A is not positive definite.  b must be null
// (the reference passes 0).
inline bool Cholesky(double* A, size_t astep, int m, double* b, size_t, int) {
  if (b) throw std::runtime_error("refpin shim: Cholesky with a right-hand side");
  const size_t s = astep / sizeof(double);
  for (int i = 0; i < m; ++i) {
    for (int j = 0; j < i; ++j) {
      double v = A[i * s + j];
      for (int k = 0; k < j; ++k) v -= A[i * s + k] * A[j * s + k];
      A[i * s + j] = v * A[j * s + j];           // the diagonal holds 1 / L_jj here
    }
    double v = A[i * s + i];
    for (int k = 0; k < i; ++k) v -= A[i * s + k] * A[i * s + k];
    if (!(v > 0.0)) return false;
    A[i * s + i] = 1.0 / std::sqrt(v);
  }
  if (cholesky_convention() == 3)
    for (int i = 0; i < m; ++i) A[i * s + i] = 1.0 / A[i * s + i];
  return true;
}

inline void log(const Mat& src, Mat& dst) {
  Mat r = src.clone();
  for (int i = 0; i < r.rows; ++i)
    for (int j = 0; j < r.cols; ++j) r.at<double>(i, j) = std::log(r.at<double>(i, j));
  dst = r;
}
inline void exp(const Mat& src, Mat& dst) {
  Mat r = src.clone();
  for (int i = 0; i < r.rows; ++i)
    for (int j = 0; j < r.cols; ++j) r.at<double>(i, j) = std::exp(r.at<double>(i, j));
  dst = r;
}
inline void pow(const Mat& src, double p, Mat& dst) {
  Mat r = src.clone();
  for (int i = 0; i < r.rows; ++i)
    for (int j = 0; j < r.cols; ++j) r.at<double>(i, j) = p == 2.0 ? r.at<double>(i, j) * r.at<double>(i, j)
                                                                   : std::pow(r.at<double>(i, j), p);
  dst = r;
}
inline Scalar sum(const Mat& m) {
  double s = 0.0;
  for (int i = 0; i < m.rows; ++i)
    for (int j = 0; j < m.cols; ++j) s += m.at<double>(i, j);
  return Scalar(s);
}
// dim 1: one column of row sums; dim 0: one row of column sums
inline void reduce(const Mat& src, Mat& dst, int dim, int, int = -1) {
  Mat r = dim == 1 ? Mat(src.rows, 1, CV_64F) : Mat(1, src.cols, CV_64F);
  for (int i = 0; i < src.rows; ++i)
    for (int j = 0; j < src.cols; ++j) {
      if (dim == 1) r.at<double>(i, 0) += src.at<double>(i, j);
      else r.at<double>(0, j) += src.at<double>(i, j);
    }
  dst = r;
}
inline Mat repeat(const Mat& src, int ny, int nx) {
  Mat r(src.rows * ny, src.cols * nx, CV_64F);
  for (int i = 0; i < r.rows; ++i)
    for (int j = 0; j < r.cols; ++j) r.at<double>(i, j) = src.at<double>(i % src.rows, j % src.cols);
  return r;
}
inline void split(const Mat& src, std::vector<Mat>& ch) {
  ch.clear();
  for (int c = 0; c < src.cn; ++c) {
    Mat m(src.rows, src.cols, CV_64F);
    for (int i = 0; i < src.rows; ++i)
      for (int j = 0; j < src.cols; ++j) m.at<double>(i, j) = src.data_[(size_t)i * src.ld() + (size_t)j * src.cn + c];
    ch.push_back(m);
  }
}
inline void vconcat(const Mat& a, const Mat& b, Mat& dst) {
  Mat r(a.rows + b.rows, a.cols, CV_64F);
  for (int i = 0; i < a.rows; ++i)
    for (int j = 0; j < a.cols; ++j) r.at<double>(i, j) = a.at<double>(i, j);
  for (int i = 0; i < b.rows; ++i)
    for (int j = 0; j < b.cols; ++j) r.at<double>(a.rows + i, j) = b.at<double>(i, j);
  dst = r;
}

// ---------------------------------------------------------------- injected draws
std::deque<double>& injected_uniforms();          // RNG::uniform(double, double): u in [0, 1)
std::deque<int>& injected_ints();                 // RNG::uniform(int, int)
std::deque<double>& injected_normals();           // randn

inline int64_t getTickCount() { return 0; }

class RNG {
 public:
  explicit RNG(uint64_t = 0) {}
  double uniform(double a, double b) {
    auto& q = injected_uniforms();
    if (q.empty()) throw std::runtime_error("refpin shim: no injected uniform left");
    const double u = q.front();
    q.pop_front();
    return a + (b - a) * u;
  }
  int uniform(int a, int b) {
    auto& q = injected_ints();
    if (q.empty()) throw std::runtime_error("refpin shim: no injected integer left");
    const int v = q.front();
    q.pop_front();
    if (v < a || v >= b) throw std::runtime_error("refpin shim: injected integer out of range");
    return v;
  }
};

// randn with a vector mean and a matrix "stddev": each element's channel
// vector is mean + stddev * n, n standard normal (injected)
inline void randn(Mat& dst, const Mat& mean, const Mat& stddev) {
  const int cn = dst.cn;
  for (int i = 0; i < dst.rows; ++i)
    for (int j = 0; j < dst.cols; ++j) {
      double n[4];
      for (int c = 0; c < cn; ++c) {
        auto& q = injected_normals();
        if (q.empty()) throw std::runtime_error("refpin shim: no injected normal left");
        n[c] = q.front();
        q.pop_front();
      }
      for (int c = 0; c < cn; ++c) {
        double v = mean.at<double>(c);
        for (int k = 0; k < cn; ++k) v += stddev.at<double>(c, k) * n[k];
        dst.data_[(size_t)i * dst.ld() + (size_t)j * cn + c] = v;
      }
    }
}

}  // namespace cv

#endif
