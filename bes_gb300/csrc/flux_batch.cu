// Per-face flux and first-order flux Jacobian for independent faces: the unit-test surface of
// Flux_<double>::computeFlux (include/Flux.hpp:43-46) and FluxJacobian::computeJacobian
// (include/FluxJacobian.hpp:39-44).  Jacobians are forward-mode derivatives of the same
// templated flux code (two passes of 5 derivative slots: left state, then right state).
#include <cstring>
#include <vector>

#include "context.hpp"

using namespace bes;

namespace {

typedef Dual<5, double> D5;

__global__ void flux_batch_kernel(GasConst g, Params prm, int kind, int64_t n,
                                  const double* __restrict__ UL, const double* __restrict__ UR,
                                  const double* __restrict__ nh, double* __restrict__ F,
                                  double* __restrict__ JL, double* __restrict__ JR) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double l[5], r[5], nn[3], f[5];
  for (int v = 0; v < 5; ++v) {
    l[v] = UL[i * 5 + v];
    r[v] = UR[i * 5 + v];
  }
  for (int d = 0; d < 3; ++d) nn[d] = nh[i * 3 + d];
  if (kind == 0)
    roe_flux(g, l, r, nn, f);
  else if (kind == 1)
    slipwall_flux(g, l, nn, f);
  else
    freestream_flux(g, l, prm.pinf, nn, f);
  for (int v = 0; v < 5; ++v) F[i * 5 + v] = f[v];
  if (!JL) return;
  for (int side = 0; side < (kind == 0 && JR ? 2 : 1); ++side) {
    D5 dl[5], dr[5], df[5];
    for (int v = 0; v < 5; ++v) {
      dl[v] = D5(l[v]);
      dr[v] = D5(r[v]);
      if (side == 0)
        dl[v].d[v] = 1.0;
      else
        dr[v].d[v] = 1.0;
    }
    if (kind == 0)
      roe_flux(g, dl, dr, nn, df);
    else if (kind == 1)
      slipwall_flux(g, dl, nn, df);
    else
      freestream_flux(g, dl, prm.pinf, nn, df);
    double* J = side == 0 ? JL : JR;
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) J[i * 25 + a * 5 + b] = df[a].d[b];
  }
}

}  // namespace

extern "C" int bes_flux_batch(bes_ctx* ctx, int32_t kind, int64_t n, const double* UL,
                              const double* UR, const double* nhat, double* F, double* JL,
                              double* JR) {
  if (!ctx || n < 0 || kind < 0 || kind > 2 || !UL || !nhat || !F) return BES_ERR_INVALID;
  if (n == 0) return BES_OK;
  std::vector<double> zeros;
  if (!UR) {
    zeros.assign(n * 5, 0.0);
    UR = zeros.data();
  }
  double *dUL, *dUR, *dn, *dF, *dJL = nullptr, *dJR = nullptr;
  const size_t s5 = n * 5 * sizeof(double), s3 = n * 3 * sizeof(double), s25 = n * 25 * sizeof(double);
  cudaError_t e = cudaMalloc(&dUL, s5);
  if (e == cudaSuccess) e = cudaMalloc(&dUR, s5);
  if (e == cudaSuccess) e = cudaMalloc(&dn, s3);
  if (e == cudaSuccess) e = cudaMalloc(&dF, s5);
  if (e == cudaSuccess && JL) e = cudaMalloc(&dJL, s25);
  if (e == cudaSuccess && JL) e = cudaMalloc(&dJR, s25);
  if (e != cudaSuccess) {
    ctx->last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return BES_ERR_CUDA;
  }
  cudaMemcpy(dUL, UL, s5, cudaMemcpyHostToDevice);
  cudaMemcpy(dUR, UR, s5, cudaMemcpyHostToDevice);
  cudaMemcpy(dn, nhat, s3, cudaMemcpyHostToDevice);
  const int threads = 128;
  flux_batch_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, ctx->stream>>>(
      ctx->prm.gas, ctx->prm, kind, n, dUL, dUR, dn, dF, dJL, kind == 0 ? dJR : nullptr);
  e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(F, dF, s5, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && JL) e = cudaMemcpy(JL, dJL, s25, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && JL && JR && kind == 0) e = cudaMemcpy(JR, dJR, s25, cudaMemcpyDeviceToHost);
  cudaFree(dUL);
  cudaFree(dUR);
  cudaFree(dn);
  cudaFree(dF);
  if (dJL) cudaFree(dJL);
  if (dJR) cudaFree(dJR);
  if (e != cudaSuccess) {
    ctx->last_error = std::string("flux batch: ") + cudaGetErrorString(e);
    return BES_ERR_CUDA;
  }
  return BES_OK;
}
