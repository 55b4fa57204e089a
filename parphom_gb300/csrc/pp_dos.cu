// Density of states from the frequencies of a q-grid: linear triangulation
// and Gaussian / Lorentzian smearing, restated from the reference's
// BZ-integration routines (Utilities/pyphutil/fortran_routines/
// bz_integration.f90:12-48, 50-65, 68-133, 154-199).
//
// Triangulation: for each energy E, triangle and band, the four values
// (E with weight 0 and the band's frequencies at the three vertices with
// their weights f) are sorted by value with the same exchange sort; the
// position E takes decides the closed-form contribution (dos, nd) of that
// triangle, with the same case order (position 4, 3, 2, 1; a later case
// overrides an earlier one when values tie).  One thread per (energy, band)
// loops over the triangles; the per-band partials are summed in a second
// pass.  FP64 throughout.
#include <cstdint>
#include <vector>

#include "../../include/parphom_gpu.h"
#include "pp_internal.cuh"

namespace {

constexpr double PI_REF = (double)3.141592653589793f;  // bz_integration.f90:185, 195

__device__ void integrate_triangle(const double a[4][2], double Ef, double &dos, double &nd) {
  dos = 0.0;
  nd = 0.0;
  if (a[3][0] == Ef) {
    dos = 0.0;
    nd = a[0][1] + a[1][1] + a[2][1];
  }
  if (a[2][0] == Ef) {
    const double e0 = a[0][0], f0 = a[0][1], e1 = a[1][0], f1 = a[1][1], e2 = a[3][0], f2 = a[3][1];
    const double del02 = (e2 - Ef) / (e2 - e0), del12 = (e2 - Ef) / (e2 - e1);
    const double ddel02 = 1 / (e0 - e2), ddel12 = 1 / (e1 - e2);
    nd = (1 - del12 * (del02 * del02)) * f0 + (1 - del02 * (del12 * del12)) * f1 +
         (1 - 3 * del12 * del02 + del12 * (del02 * del02) + del02 * (del12 * del12)) * f2;
    dos = (-2 * del02 * ddel02 * del12 - ddel12 * (del02 * del02)) * f0 +
          (-ddel02 * (del12 * del12) - 2 * del02 * del12 * ddel12) * f1 +
          (-3 * del12 * ddel02 - 3 * del02 * ddel12 + 2 * del02 * del12 * ddel02 + ddel12 * (del02 * del02) +
           2 * del02 * del12 * ddel12 + ddel02 * (del12 * del12)) *
              f2;
  }
  if (a[1][0] == Ef) {
    const double e0 = a[0][0], f0 = a[0][1], e1 = a[2][0], f1 = a[2][1], e2 = a[3][0], f2 = a[3][1];
    const double del10 = (Ef - e0) / (e1 - e0), del20 = (Ef - e0) / (e2 - e0);
    const double ddel10 = 1 / (e1 - e0), ddel20 = 1 / (e2 - e0);
    double n = (3 - del10 - del20) * f0 + del10 * f1 + del20 * f2;
    dos = ddel10 * del20 * n + del10 * ddel20 * n + del10 * del20 * ((-ddel10 - ddel20) * f0 + ddel10 * f1 + ddel20 * f2);
    nd = n * del10 * del20;
  }
  if (a[0][0] == Ef) {
    dos = 0.0;
    nd = 0.0;
  }
}

__global__ void k_dos_tri(const double *freq, const double *func, int64_t ldf, int64_t nbands, const int64_t *tri,
                          int64_t ntri, const double *E, int64_t ne, double *pdos, double *pnd) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // band
  const int64_t i = blockIdx.y;                                      // energy
  if (k >= nbands || i >= ne) return;
  const double Ef = E[i];
  double sd = 0.0, sn = 0.0;
  for (int64_t j = 0; j < ntri; ++j) {
    double a[4][2];
    a[0][0] = Ef;
    a[0][1] = 0.0;
    for (int v = 0; v < 3; ++v) {
      const int64_t q = tri[3 * j + v];
      a[v + 1][0] = freq[q * ldf + k];
      a[v + 1][1] = func ? func[q * ldf + k] : 1.0;
    }
    for (int p = 0; p < 4; ++p)  // exchange sort of bz_integration.f90:50-65
      for (int r = p + 1; r < 4; ++r)
        if (a[p][0] > a[r][0]) {
          const double t0 = a[p][0], t1 = a[p][1];
          a[p][0] = a[r][0];
          a[p][1] = a[r][1];
          a[r][0] = t0;
          a[r][1] = t1;
        }
    double d, n;
    integrate_triangle(a, Ef, d, n);
    sd += d;
    sn += n;
  }
  pdos[i * nbands + k] = sd;
  pnd[i * nbands + k] = sn;
}

__global__ void k_dos_smear(int method, const double *freq, int64_t ldf, int64_t nq, int64_t nbands,
                            const double *weights, double width, const double *E, int64_t ne, double *pdos) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // band
  const int64_t i = blockIdx.y;
  if (k >= nbands || i >= ne) return;
  const double e = E[i];
  double s = 0.0;
  for (int64_t q = 0; q < nq; ++q) {
    const double e0 = freq[q * ldf + k];
    double d;
    if (method == 1) {
      const double x = (e - e0) / width;
      d = exp(-(x * x) / 2) / (sqrt(2 * PI_REF) * width);
    } else {
      const double h = width / 2;
      d = (h / ((e - e0) * (e - e0) + h * h)) * (1 / PI_REF);
    }
    s += d * weights[q];
  }
  pdos[i * nbands + k] = s;
}

__global__ void k_sum_rows(const double *p, int64_t ne, int64_t nb, double scale, double *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ne) return;
  double s = 0.0;
  for (int64_t k = 0; k < nb; ++k) s += p[i * nb + k];
  out[i] = s * scale;
}

int cerr(cudaError_t e) { return e == cudaSuccess ? PP_OK : (e == cudaErrorMemoryAllocation ? PP_ERR_NOMEM : PP_ERR_CUDA); }

// ---- device-resident forms: every array in device memory, no scratch.
// One thread per band, one block row per energy; the block's bands are
// summed in shared memory and added to the energy's total (zeroed first).
constexpr int DV_NT = 128;

__device__ __forceinline__ double block_sum128(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < DV_NT / 32; ++k) r += sh[k];
  return r;  // valid in thread 0
}

__global__ void __launch_bounds__(DV_NT) k_dos_tri_dev(const double *freq, int64_t ldf, const double *func,
                                                       int64_t ldfunc, int64_t nbands, const int64_t *tri,
                                                       int64_t ntri, const double *E, int64_t ne, double *dos,
                                                       double *nd) {
  __shared__ double sh[2][DV_NT / 32];
  const int64_t k = (int64_t)blockIdx.x * DV_NT + threadIdx.x;  // band
  const int64_t i = blockIdx.y;                                 // energy
  if (i >= ne) return;
  const double Ef = E[i];
  double sd = 0.0, sn = 0.0;
  if (k < nbands) {
    for (int64_t j = 0; j < ntri; ++j) {
      double a[4][2];
      a[0][0] = Ef;
      a[0][1] = 0.0;
      for (int v = 0; v < 3; ++v) {
        const int64_t q = tri[3 * j + v];
        a[v + 1][0] = freq[q * ldf + k];
        a[v + 1][1] = func ? func[q * ldfunc + k] : 1.0;
      }
      for (int p = 0; p < 4; ++p)  // exchange sort of bz_integration.f90:50-65
        for (int r = p + 1; r < 4; ++r)
          if (a[p][0] > a[r][0]) {
            const double t0 = a[p][0], t1 = a[p][1];
            a[p][0] = a[r][0];
            a[p][1] = a[r][1];
            a[r][0] = t0;
            a[r][1] = t1;
          }
      double d, n;
      integrate_triangle(a, Ef, d, n);
      sd += d;
      sn += n;
    }
  }
  sd = block_sum128(sd, sh[0]);
  sn = block_sum128(sn, sh[1]);
  if (threadIdx.x == 0) {
    atomicAdd(&dos[i], sd);
    atomicAdd(&nd[i], sn);
  }
}

__global__ void __launch_bounds__(DV_NT) k_dos_smear_dev(int method, const double *freq, int64_t ldf, int64_t nq,
                                                         int64_t nbands, const double *weights, double width,
                                                         const double *E, int64_t ne, double scale, double *dos) {
  __shared__ double sh[DV_NT / 32];
  const int64_t k = (int64_t)blockIdx.x * DV_NT + threadIdx.x;
  const int64_t i = blockIdx.y;
  if (i >= ne) return;
  const double e = E[i];
  double s = 0.0;
  if (k < nbands) {
    for (int64_t q = 0; q < nq; ++q) {
      const double e0 = freq[q * ldf + k];
      double d;
      if (method == 1) {
        const double x = (e - e0) / width;
        d = exp(-(x * x) / 2) / (sqrt(2 * PI_REF) * width);
      } else {
        const double h = width / 2;
        d = (h / ((e - e0) * (e - e0) + h * h)) * (1 / PI_REF);
      }
      s += d * weights[q];
    }
  }
  s = block_sum128(s, sh);
  if (threadIdx.x == 0) atomicAdd(&dos[i], s * scale);
}

// func[q ldfunc + j] = v_a v_b of mode j at q-point q (a = b = -1: |v|^2),
// from the velocity output vel[q velstride + 3 j + d].
__global__ void k_vel_weights(const double *vel, int64_t velstride, int64_t nq, int64_t nbands, int a, int b,
                              double *func, int64_t ldfunc) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t q = blockIdx.y;
  if (j >= nbands || q >= nq) return;
  const double *v = vel + q * velstride + 3 * j;
  func[q * ldfunc + j] = (a < 0) ? v[0] * v[0] + v[1] * v[1] + v[2] * v[2] : v[a] * v[b];
}

}  // namespace

extern "C" PP_API int pp_dos_triangulation(const double *freq, int64_t ldf, int64_t nk, int64_t nbands,
                                           const double *func, const int64_t *tri, int64_t ntri, const double *energy,
                                           int64_t ne, double *dos, double *nd) {
  if (!freq) return -1;
  if (ldf < nbands) return -2;
  if (nk < 1) return -3;
  if (nbands < 1) return -4;
  if (!tri && ntri > 0) return -6;
  if (ntri < 0) return -7;
  if (!energy && ne > 0) return -8;
  if (ne < 0) return -9;
  if (!dos) return -10;
  if (!nd) return -11;
  for (int64_t j = 0; j < 3 * ntri; ++j)
    if (tri[j] < 0 || tri[j] >= nk) return -6;
  if (ne == 0) return PP_OK;
  double *dfreq = nullptr, *dfunc = nullptr, *dE = nullptr, *pd = nullptr, *pn = nullptr, *od = nullptr, *on = nullptr;
  int64_t *dtri = nullptr;
  cudaError_t e = cudaSuccess;
  auto al = [&](void **p, size_t b) {
    if (e == cudaSuccess) e = cudaMalloc(p, b > 0 ? b : 8);
  };
  al((void **)&dfreq, sizeof(double) * nk * ldf);
  if (func) al((void **)&dfunc, sizeof(double) * nk * ldf);
  al((void **)&dtri, sizeof(int64_t) * 3 * ntri);
  al((void **)&dE, sizeof(double) * ne);
  al((void **)&pd, sizeof(double) * ne * nbands);
  al((void **)&pn, sizeof(double) * ne * nbands);
  al((void **)&od, sizeof(double) * ne);
  al((void **)&on, sizeof(double) * ne);
  if (e == cudaSuccess) e = cudaMemcpy(dfreq, freq, sizeof(double) * nk * ldf, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && func) e = cudaMemcpy(dfunc, func, sizeof(double) * nk * ldf, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ntri) e = cudaMemcpy(dtri, tri, sizeof(int64_t) * 3 * ntri, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dE, energy, sizeof(double) * ne, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_dos_tri<<<dim3((unsigned)((nbands + 127) / 128), (unsigned)ne), 128>>>(dfreq, dfunc, ldf, nbands, dtri, ntri, dE,
                                                                            ne, pd, pn);
    k_sum_rows<<<(unsigned)((ne + 127) / 128), 128>>>(pd, ne, nbands, 1.0, od);
    k_sum_rows<<<(unsigned)((ne + 127) / 128), 128>>>(pn, ne, nbands, 1.0, on);
    pp::count_launch(3);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(dos, od, sizeof(double) * ne, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(nd, on, sizeof(double) * ne, cudaMemcpyDeviceToHost);
  for (void *p : {(void *)dfreq, (void *)dfunc, (void *)dtri, (void *)dE, (void *)pd, (void *)pn, (void *)od, (void *)on})
    if (p) cudaFree(p);
  return cerr(e);
}

extern "C" PP_API int pp_dos_smearing(int32_t method, const double *freq, int64_t ldf, int64_t nq, int64_t nbands,
                                      const double *weights, double width, const double *energy, int64_t ne,
                                      int64_t natom, double *dos) {
  if (method != 1 && method != 2) return -1;
  if (!freq) return -2;
  if (ldf < nbands) return -3;
  if (nq < 1) return -4;
  if (nbands < 1) return -5;
  if (!weights) return -6;
  if (!(width > 0.0)) return -7;
  if (!energy && ne > 0) return -8;
  if (ne < 0) return -9;
  if (natom < 1) return -10;
  if (!dos) return -11;
  if (ne == 0) return PP_OK;
  double *dfreq = nullptr, *dw = nullptr, *dE = nullptr, *pd = nullptr, *od = nullptr;
  cudaError_t e = cudaSuccess;
  auto al = [&](void **p, size_t b) {
    if (e == cudaSuccess) e = cudaMalloc(p, b);
  };
  al((void **)&dfreq, sizeof(double) * nq * ldf);
  al((void **)&dw, sizeof(double) * nq);
  al((void **)&dE, sizeof(double) * ne);
  al((void **)&pd, sizeof(double) * ne * nbands);
  al((void **)&od, sizeof(double) * ne);
  if (e == cudaSuccess) e = cudaMemcpy(dfreq, freq, sizeof(double) * nq * ldf, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dw, weights, sizeof(double) * nq, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dE, energy, sizeof(double) * ne, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_dos_smear<<<dim3((unsigned)((nbands + 127) / 128), (unsigned)ne), 128>>>(method, dfreq, ldf, nq, nbands, dw,
                                                                              width, dE, ne, pd);
    k_sum_rows<<<(unsigned)((ne + 127) / 128), 128>>>(pd, ne, nbands, 1.0 / (double)natom, od);
    pp::count_launch(2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(dos, od, sizeof(double) * ne, cudaMemcpyDeviceToHost);
  for (void *p : {(void *)dfreq, (void *)dw, (void *)dE, (void *)pd, (void *)od})
    if (p) cudaFree(p);
  return cerr(e);
}

extern "C" PP_API int pp_dos_triangulation_device(const double *freq_dev, int64_t ldf, int64_t nk, int64_t nbands,
                                                  const double *func_dev, int64_t ldfunc, const int64_t *tri_dev,
                                                  int64_t ntri, const double *energy_dev, int64_t ne, double *dos_dev,
                                                  double *nd_dev, void *stream) {
  if (!freq_dev) return -1;
  if (ldf < nbands) return -2;
  if (nk < 1) return -3;
  if (nbands < 1) return -4;
  if (func_dev && ldfunc < nbands) return -6;
  if (!tri_dev && ntri > 0) return -7;
  if (ntri < 0) return -8;
  if (!energy_dev && ne > 0) return -9;
  if (ne < 0) return -10;
  if (!dos_dev) return -11;
  if (!nd_dev) return -12;
  if (ne == 0) return PP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(dos_dev, 0, sizeof(double) * ne, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(nd_dev, 0, sizeof(double) * ne, s);
  if (e == cudaSuccess) {
    k_dos_tri_dev<<<dim3((unsigned)((nbands + DV_NT - 1) / DV_NT), (unsigned)ne), DV_NT, 0, s>>>(
        freq_dev, ldf, func_dev, ldfunc, nbands, tri_dev, ntri, energy_dev, ne, dos_dev, nd_dev);
    pp::count_launch(1);
    e = cudaGetLastError();
  }
  return cerr(e);
}

extern "C" PP_API int pp_dos_smearing_device(int32_t method, const double *freq_dev, int64_t ldf, int64_t nq,
                                             int64_t nbands, const double *weights_dev, double width,
                                             const double *energy_dev, int64_t ne, int64_t natom, double *dos_dev,
                                             void *stream) {
  if (method != 1 && method != 2) return -1;
  if (!freq_dev) return -2;
  if (ldf < nbands) return -3;
  if (nq < 1) return -4;
  if (nbands < 1) return -5;
  if (!weights_dev) return -6;
  if (!(width > 0.0)) return -7;
  if (!energy_dev && ne > 0) return -8;
  if (ne < 0) return -9;
  if (natom < 1) return -10;
  if (!dos_dev) return -11;
  if (ne == 0) return PP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(dos_dev, 0, sizeof(double) * ne, s);
  if (e == cudaSuccess) {
    k_dos_smear_dev<<<dim3((unsigned)((nbands + DV_NT - 1) / DV_NT), (unsigned)ne), DV_NT, 0, s>>>(
        method, freq_dev, ldf, nq, nbands, weights_dev, width, energy_dev, ne, 1.0 / (double)natom, dos_dev);
    pp::count_launch(1);
    e = cudaGetLastError();
  }
  return cerr(e);
}

extern "C" PP_API int pp_velocity_weights_device(const double *vel_dev, int64_t velstride, int64_t nq, int64_t nbands,
                                                 int32_t a, int32_t b, double *func_dev, int64_t ldfunc,
                                                 void *stream) {
  if (!vel_dev) return -1;
  if (velstride < 3 * nbands) return -2;
  if (nq < 0) return -3;
  if (nbands < 1) return -4;
  if (!((a == -1 && b == -1) || (a >= 0 && a < 3 && b >= 0 && b < 3))) return -5;
  if (!func_dev) return -7;
  if (ldfunc < nbands) return -8;
  if (nq == 0) return PP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  k_vel_weights<<<dim3((unsigned)((nbands + 127) / 128), (unsigned)nq), 128, 0, s>>>(vel_dev, velstride, nq, nbands,
                                                                                     a, b, func_dev, ldfunc);
  pp::count_launch(1);
  return cerr(cudaGetLastError());
}
