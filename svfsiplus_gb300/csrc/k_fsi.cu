// Generalised-alpha state updates of the coupled FSI time step (pic.cpp:74-767 with two
// equations): the state arrays hold 7 rows per node, rows 0..3 for the FSI equation
// (first order: velocity, pressure; displacement rows 0..2 on solid nodes) and rows
// 4..6 for the mesh-motion equation (second order: mesh displacement).  Each row uses
// the generalised-alpha constants of its equation.
//
// The arithmetic is written with explicit round-to-nearest operations in the
// reference's evaluation order (no fused multiply-add), so these streaming updates
// give the reference's values bit for bit.
#include "internal.h"

namespace svgpu {

namespace {

constexpr int kRows = 7;

__device__ __forceinline__ int eq_of_row(int r) { return r < 4 ? 0 : 1; }

// picp (pic.cpp:591-767) with dFlag and no sstEq: An = Ao (gam-1)/gam, Yn = Yo,
// Dn = (Do + Yn dt) + An dt^2 (gam/2 - beta)/(gam - 1), per equation.
__global__ void fsi_predict_kernel(long n7, FsiCoefs c, const double* __restrict__ Ao, const double* __restrict__ Yo,
                                   const double* __restrict__ Do, double* __restrict__ An, double* __restrict__ Yn,
                                   double* __restrict__ Dn) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n7; i += (long)gridDim.x * blockDim.x) {
    const int q = eq_of_row((int)(i % kRows));
    const double a = __dmul_rn(Ao[i], c.pred_a[q]);
    const double y = Yo[i];
    An[i] = a;
    Yn[i] = y;
    Dn[i] = __dadd_rn(__dadd_rn(Do[i], __dmul_rn(y, c.dt)), __dmul_rn(a, c.pred_d[q]));
  }
}

// Strong Dirichlet values of one equation: rows s..s+2 of the listed nodes.
__global__ void fsi_dirichlet_kernel(int n, int s, const int* __restrict__ nodes, const double* __restrict__ dirY,
                                     const double* __restrict__ dirA, double* __restrict__ An, double* __restrict__ Yn) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long a = nodes[k];
  for (int i = 0; i < 3; i++) {
    An[kRows * a + s + i] = dirA[3L * k + i];
    Yn[kRows * a + s + i] = dirY[3L * k + i];
  }
}

// pici (pic.cpp:486-589) for every equation: Ag = Ao (1-am) + An am,
// Yg = Yo (1-af) + Yn af, Dg = Do (1-af) + Dn af.
__global__ void fsi_initiate_kernel(long n7, FsiCoefs c, const double* __restrict__ Ao, const double* __restrict__ An,
                                    const double* __restrict__ Yo, const double* __restrict__ Yn,
                                    const double* __restrict__ Do, const double* __restrict__ Dn,
                                    double* __restrict__ Ag, double* __restrict__ Yg, double* __restrict__ Dg) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n7; i += (long)gridDim.x * blockDim.x) {
    const int q = eq_of_row((int)(i % kRows));
    Ag[i] = __dadd_rn(__dmul_rn(Ao[i], c.ini[q][0]), __dmul_rn(An[i], c.ini[q][1]));
    Yg[i] = __dadd_rn(__dmul_rn(Yo[i], c.ini[q][2]), __dmul_rn(Yn[i], c.ini[q][3]));
    Dg[i] = __dadd_rn(__dmul_rn(Do[i], c.ini[q][2]), __dmul_rn(Dn[i], c.ini[q][3]));
  }
}

// picc (pic.cpp:74-329) after a solve of the FSI equation: rows 0..3 take the
// increment R (4, nNo); then every node of a solid domain copies its rows 0..2 of An,
// Yn, Dn into the mesh rows 4..6 (pic.cpp:181-201).
__global__ void fsi_correct_kernel(int nNo, double c0, double c1, const double* __restrict__ R,
                                   const uint8_t* __restrict__ solid, double* __restrict__ An, double* __restrict__ Yn,
                                   double* __restrict__ Dn) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nNo) return;
  double* an = An + (long)kRows * a;
  double* yn = Yn + (long)kRows * a;
  double* dn = Dn + (long)kRows * a;
  for (int i = 0; i < 4; i++) {
    const double r = R[4L * a + i];
    an[i] = __dsub_rn(an[i], r);
    yn[i] = __dsub_rn(yn[i], __dmul_rn(r, c0));
    dn[i] = __dsub_rn(dn[i], __dmul_rn(r, c1));
  }
  if (solid[a]) {
    for (int i = 0; i < 3; i++) {
      an[4 + i] = an[i];
      yn[4 + i] = yn[i];
      dn[4 + i] = dn[i];
    }
  }
}

// picc after a solve of the mesh equation: rows 4..6 take the increment R (3, nNo).
__global__ void mesh_correct_kernel(int nNo, double c0, double c1, const double* __restrict__ R,
                                    double* __restrict__ An, double* __restrict__ Yn, double* __restrict__ Dn) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nNo) return;
  for (int i = 0; i < 3; i++) {
    const double r = R[3L * a + i];
    const long k = (long)kRows * a + 4 + i;
    An[k] = __dsub_rn(An[k], r);
    Yn[k] = __dsub_rn(Yn[k], __dmul_rn(r, c0));
    Dn[k] = __dsub_rn(Dn[k], __dmul_rn(r, c1));
  }
}

// The mesh equation's dof-3 system embedded in 4x4 blocks for the mixed-precision
// multilevel solver: each 3x3 block in the upper left, a fourth unknown that only its
// own unit diagonal touches (zero right-hand side, zero solution).
__global__ void pad_mesh_matrix_kernel(long nnz, const int* __restrict__ blkRow, const int* __restrict__ colPtr,
                                       const double* __restrict__ Val9, float* __restrict__ Val16) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const double* a = Val9 + 9 * k;
  float4* o = reinterpret_cast<float4*>(Val16 + 16 * k);
  const float d = blkRow[k] == colPtr[k] ? 1.f : 0.f;
  o[0] = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
  o[1] = make_float4((float)a[3], (float)a[4], (float)a[5], 0.f);
  o[2] = make_float4((float)a[6], (float)a[7], (float)a[8], 0.f);
  o[3] = make_float4(0.f, 0.f, 0.f, d);
}

__global__ void pad_vec_kernel(int nNo, const double* __restrict__ R3, double* __restrict__ R4) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nNo) return;
  R4[4L * a] = R3[3L * a];
  R4[4L * a + 1] = R3[3L * a + 1];
  R4[4L * a + 2] = R3[3L * a + 2];
  R4[4L * a + 3] = 0.0;
}

__global__ void unpad_vec_kernel(int nNo, const double* __restrict__ R4, double* __restrict__ R3) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nNo) return;
  R3[3L * a] = R4[4L * a];
  R3[3L * a + 1] = R4[4L * a + 1];
  R3[3L * a + 2] = R4[4L * a + 2];
}

}  // namespace

void launch_pad_mesh_system(cudaStream_t s, int nNo, long nnz, const int* blkRow, const int* colPtr,
                            const double* Val9, const double* R3, float* Val16, double* R4) {
  if (Val9) pad_mesh_matrix_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, blkRow, colPtr, Val9, Val16);
  pad_vec_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, R3, R4);
}

void launch_unpad_vec(cudaStream_t s, int nNo, const double* R4, double* R3) {
  unpad_vec_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, R4, R3);
}

void launch_fsi_predict(cudaStream_t s, int nNo, const FsiCoefs& c, const double* Ao, const double* Yo,
                        const double* Do, double* An, double* Yn, double* Dn) {
  const long n7 = (long)kRows * nNo;
  fsi_predict_kernel<<<grid_for(n7, 256), 256, 0, s>>>(n7, c, Ao, Yo, Do, An, Yn, Dn);
}

void launch_fsi_dirichlet(cudaStream_t s, int n, int row0, const int* nodes, const double* dirY, const double* dirA,
                          double* An, double* Yn) {
  if (n <= 0) return;
  fsi_dirichlet_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, row0, nodes, dirY, dirA, An, Yn);
}

void launch_fsi_initiate(cudaStream_t s, int nNo, const FsiCoefs& c, const double* Ao, const double* An,
                         const double* Yo, const double* Yn, const double* Do, const double* Dn, double* Ag,
                         double* Yg, double* Dg) {
  const long n7 = (long)kRows * nNo;
  fsi_initiate_kernel<<<grid_for(n7, 256), 256, 0, s>>>(n7, c, Ao, An, Yo, Yn, Do, Dn, Ag, Yg, Dg);
}

void launch_fsi_correct(cudaStream_t s, int nNo, double c0, double c1, const double* R, const uint8_t* solid,
                        double* An, double* Yn, double* Dn) {
  fsi_correct_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, c0, c1, R, solid, An, Yn, Dn);
}

void launch_mesh_correct(cudaStream_t s, int nNo, double c0, double c1, const double* R, double* An, double* Yn,
                         double* Dn) {
  mesh_correct_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, c0, c1, R, An, Yn, Dn);
}

}  // namespace svgpu
