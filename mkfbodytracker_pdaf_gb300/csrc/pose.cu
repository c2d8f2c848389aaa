// pose.cu -- batched pose decode and 3-D back-projection (the step after the
// estimate): e = Hpca^T x + mpca (pfPose.cpp:347-348), get3Dpose
// (pfPose.cpp:93-127) and the publish2Dpos point record (pfPose.cpp:173-208).
// FP64, one thread per estimate; Hpca and mpca staged in shared memory.
#include "mkf_common.cuh"

namespace mkf {

constexpr int kPoseMaxF = 64;
constexpr int kPoseTB = 128;

// 3x3 inverse by Gauss-Jordan elimination with partial pivoting (DECOMP_LU)
__device__ bool inv3(const double* A, double* Ai) {
  double M[3][6];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 6; ++c) M[r][c] = c < 3 ? A[r * 3 + c] : (c - 3 == r ? 1.0 : 0.0);
  for (int c = 0; c < 3; ++c) {
    int piv = c;
    double best = fabs(M[c][c]);
    for (int r = c + 1; r < 3; ++r)
      if (fabs(M[r][c]) > best) { best = fabs(M[r][c]); piv = r; }
    if (best == 0.0 || !isfinite(best)) return false;
    if (piv != c)
      for (int k = 0; k < 6; ++k) { double t = M[c][k]; M[c][k] = M[piv][k]; M[piv][k] = t; }
    const double inv = 1.0 / M[c][c];
    for (int k = 0; k < 6; ++k) M[c][k] *= inv;
    for (int r = 0; r < 3; ++r) {
      if (r == c) continue;
      const double f = M[r][c];
      for (int k = 0; k < 6; ++k) M[r][k] -= f * M[c][k];
    }
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Ai[r * 3 + c] = M[r][c + 3];
  return true;
}

struct PoseArgs {
  const double* x;
  int B, d, F;
  const double *Hpca, *mpca;
  double Kc[9];
  double* e_out;
  double* pos3d;
  int* status;
};

__global__ void __launch_bounds__(kPoseTB) pose_decode_kernel(PoseArgs A) {
  extern __shared__ double s_pose[];
  double* sH = s_pose;                       // d x F
  double* sm = s_pose + A.d * A.F;           // F
  for (int q = threadIdx.x; q < A.d * A.F; q += blockDim.x) sH[q] = A.Hpca[q];
  for (int q = threadIdx.x; q < A.F; q += blockDim.x) sm[q] = A.mpca[q];
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= A.B) return;
  const double* x = A.x + (size_t)b * A.d;
  double e[kPoseMaxF];
  for (int f = 0; f < A.F; ++f) {
    double s = 0.0;
    for (int r = 0; r < A.d; ++r) s += sH[r * A.F + f] * x[r];
    e[f] = s + sm[f];
    if (A.e_out) A.e_out[(size_t)b * A.F + f] = e[f];
  }
  if (!A.pos3d) return;
  const double roll = e[16], pitch = e[17], yaw = e[15];
  double sr, cr, sp, cp, sy, cy;
  sincos(roll, &sr, &cr);
  sincos(pitch, &sp, &cp);
  sincos(yaw, &sy, &cy);
  // R = R3(yaw) R2(pitch) R1(roll)
  const double R[9] = {cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr,
                       sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr,
                       -sp, cp * sr, cp * cr};
  double P3[9], Pi[9], p4[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      P3[i * 3 + j] = A.Kc[i * 3 + 0] * R[0 * 3 + j] + A.Kc[i * 3 + 1] * R[1 * 3 + j] + A.Kc[i * 3 + 2] * R[2 * 3 + j];
    p4[i] = A.Kc[i * 3 + 0] * e[18] + A.Kc[i * 3 + 1] * e[19] + A.Kc[i * 3 + 2] * e[20];
  }
  double* out = A.pos3d + (size_t)b * 15;
  if (!inv3(P3, Pi)) {
    atomicOr(A.status, MKF_ST_NONPD);
    for (int q = 0; q < 15; ++q) out[q] = NAN;
    return;
  }
  for (int k = 0; k < 5; ++k) {
    const double Z = e[3 * k + 2];
    const double ip0 = e[3 * k] * Z - p4[0], ip1 = e[3 * k + 1] * Z - p4[1], ip2 = Z - p4[2];
    for (int i = 0; i < 3; ++i) out[i * 5 + k] = Pi[i * 3 + 0] * ip0 + Pi[i * 3 + 1] * ip1 + Pi[i * 3 + 2] * ip2;
  }
}

__global__ void pose2d_record_kernel(const double* e1, const double* e2, int B, int F, double* pts) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const double* a = e1 + (size_t)b * F;
  const double* c = e2 + (size_t)b * F;
  double* p = pts + (size_t)b * 16;
  p[0] = a[0]; p[1] = a[1];
  p[2] = c[0]; p[3] = c[1];
  p[4] = 0.5 * (a[9] + c[9]); p[5] = 0.5 * (a[10] + c[10]);
  p[6] = 0.5 * (a[12] + c[12]); p[7] = 0.5 * (a[13] + c[13]);
  p[8] = a[3]; p[9] = a[4];
  p[10] = c[3]; p[11] = c[4];
  p[12] = a[6]; p[13] = a[7];
  p[14] = c[6]; p[15] = c[7];
}

}  // namespace mkf

using namespace mkf;

extern "C" int mkf_pose_decode(const double* d_x, int B, int d, int F, const double* d_Hpca, const double* d_mpca,
                               const double* Kc, double* d_e, double* d_pos3d, int* d_status, mkf_stream_t stream) {
  MKF_RANGE("mkf_pose_decode");
  MKF_ARG(B >= 0 && d >= 1 && d <= MKF_MAX_D && F >= 1 && F <= kPoseMaxF,
          "mkf_pose_decode: bad argument (B >= 0, 1 <= d <= 24, 1 <= F <= 64)");
  if (B == 0) return MKF_OK;
  MKF_ARG(d_x && d_Hpca && d_mpca, "mkf_pose_decode: null argument");
  MKF_ARG(!d_pos3d || (F >= 21 && Kc && d_status), "mkf_pose_decode: the 3-D pose needs F >= 21, Kc and d_status");
  PoseArgs a;
  a.x = d_x; a.B = B; a.d = d; a.F = F; a.Hpca = d_Hpca; a.mpca = d_mpca;
  for (int q = 0; q < 9; ++q) a.Kc[q] = Kc ? Kc[q] : 0.0;
  a.e_out = d_e; a.pos3d = d_pos3d; a.status = d_status;
  const size_t smem = sizeof(double) * (size_t)(d * F + F);
  pose_decode_kernel<<<(B + kPoseTB - 1) / kPoseTB, kPoseTB, smem, (cudaStream_t)stream>>>(a);
  MKF_CHECK_LAUNCH("mkf_pose_decode");
  return MKF_OK;
}

extern "C" int mkf_pose2d_record(const double* d_e1, const double* d_e2, int B, int F, double* d_pts,
                                 mkf_stream_t stream) {
  MKF_ARG(B >= 0 && F >= 14, "mkf_pose2d_record: bad argument (B >= 0, F >= 14)");
  if (B == 0) return MKF_OK;
  MKF_ARG(d_e1 && d_e2 && d_pts, "mkf_pose2d_record: null argument");
  pose2d_record_kernel<<<(B + 127) / 128, 128, 0, (cudaStream_t)stream>>>(d_e1, d_e2, B, F, d_pts);
  MKF_CHECK_LAUNCH("mkf_pose2d_record");
  return MKF_OK;
}
