// transport_upwind.cu -- transport of the time-stepped operator-split run:
// explicit first-order upwind sub-steps of the aqueous totals on a
// structured grid of unit cells, the scheme of RTExplicitAdvection with
// TVD_LIMITER_UPWIND (src/pflotran/reactive_transport.F90:4501-4863,
// transport.F90:958-1043).  Built into its own library: the chemistry
// library's boundary is the reaction step, this kernel only keeps the run's
// transport on the GPU inside the step's graph.
//
// The flow field is steady, so the upwind update of a cell is a fixed
// non-negative combination of its own and its upstream neighbours' totals:
//   T'[c] = a0 T[c] + aw Tw[c] + ae Te[c] + as Ts[c] + an Tn[c] + ab Tb[c] + at Tt[c]
// with a0 = 1 - (dt_sub / V_pore) * (outgoing face flux) and a_f =
// (dt_sub / V_pore) * (incoming flux through face f), 0 for outgoing and
// closed faces.  The west neighbour of an x = 0 cell is the inflow water.
// The coefficients are computed once per run; a sub-step then costs one
// multiply and six FMAs per cell and component on the FP64 pipe, which on
// this part bounds the kernel before HBM does.
//
// Layout: T[c][x][y][z] (c slowest, z fastest); coef[k][x][y][z], k = a0,
// aw, ae, as, an, ab, at.
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) upwind_step(const double *__restrict__ T, double *__restrict__ Tn,
                                                   const double *__restrict__ coef,
                                                   const double *__restrict__ inflow, int ncomp, int nx, int ny,
                                                   int nz) {
  const long long n = (long long)nx * ny * nz;
  const long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (cell >= n) return;
  const long long sx = (long long)ny * nz, sy = nz;
  const int z = (int)(cell % nz);
  const int y = (int)((cell / nz) % ny);
  const int x = (int)(cell / sx);
  double a[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) a[k] = coef[k * n + cell];
  // neighbour offsets; a missing neighbour (closed face) reads the cell
  // itself under a zero coefficient
  const long long ow = x > 0 ? -sx : 0, oe = x < nx - 1 ? sx : 0;
  const long long os = y > 0 ? -sy : 0, on = y < ny - 1 ? sy : 0;
  const long long ob = z > 0 ? -1 : 0, ot = z < nz - 1 ? 1 : 0;
  const bool west_inflow = x == 0;
  for (int c = 0; c < ncomp; ++c) {
    const double *Tc = T + c * n + cell;
    double acc = a[0] * Tc[0];
    const double tw = Tc[ow];
    acc = fma(a[1], west_inflow ? inflow[c] : tw, acc);
    acc = fma(a[2], Tc[oe], acc);
    acc = fma(a[3], Tc[os], acc);
    acc = fma(a[4], Tc[on], acc);
    acc = fma(a[5], Tc[ob], acc);
    acc = fma(a[6], Tc[ot], acc);
    Tn[c * n + cell] = acc;
  }
}

}  // namespace

extern "C" {

// `nsub` upwind sub-steps from T0 into T1 (tmp: scratch of the same size;
// T0 is not written), with the per-cell coefficients `coef` [7][nx][ny][nz]
// and the inflow composition `inflow` [ncomp].  Enqueued on `stream` (a
// cudaStream_t) without synchronisation, so it can be captured into a
// graph; returns a cudaError_t.
int pfchem_transport_upwind(const double *T0, double *T1, double *tmp, const double *coef, const double *inflow,
                            int ncomp, int nx, int ny, int nz, int nsub, void *stream) {
  if (ncomp <= 0 || nx <= 0 || ny <= 0 || nz <= 0 || nsub <= 0) return (int)cudaErrorInvalidValue;
  if (T1 == tmp || T0 == T1 || T0 == tmp) return (int)cudaErrorInvalidValue;
  const long long n = (long long)nx * ny * nz;
  const unsigned grid = (unsigned)((n + 255) / 256);
  cudaStream_t st = (cudaStream_t)stream;
  const double *src = T0;
  for (int s = 0; s < nsub; ++s) {
    // the last sub-step lands in T1
    double *dst = ((nsub - s) & 1) ? T1 : tmp;
    upwind_step<<<grid, 256, 0, st>>>(src, dst, coef, inflow, ncomp, nx, ny, nz);
    src = dst;
  }
  return (int)cudaGetLastError();
}
}
