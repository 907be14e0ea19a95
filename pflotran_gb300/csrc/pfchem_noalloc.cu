// pfchem_noalloc.cu -- pfchem_react_batch_noalloc: the batched reaction step
// for callers that cannot allocate device memory.
//
// Some host codes own every byte of device memory through their own pool or
// arena (a PETSc or Kokkos memory pool, a coupling framework that hands out
// buffers), or call the chemistry inside a time-step loop where cudaMalloc's
// implicit device synchronisation is not acceptable.  Such a caller cannot
// create a context (pfchem_create allocates the work queue, staging buffers
// and events).  This entry point needs none of that: the caller passes the
// network, the options and device pointers for every per-cell array; the
// only global memory the solve uses beyond those -- the work-queue head and
// one statistics slot per thread block -- lives in the file-scope array
// g_noalloc_scratch below, of PFCHEM_NOALLOC_SCRATCH_BYTES bytes, which every
// GPU that loads the library keeps until the process exits.
//
// Behaviour:
//  * the first call on a device looks up the device address of the array
//    with cudaGetSymbolAddress (once per device, with that device current);
//  * every call ends by copying the statistics slots into host memory and
//    synchronising the stream, so it blocks until its solve is done and can
//    never be captured into a CUDA graph (graph users call
//    pfchem_react_batch_async on a context instead);
//  * every call shares the one array and zeroes the part it uses before the
//    launch; calls whose work overlaps on the GPU (two streams, two host
//    threads on one device) race on it, so serialise them.  Host threads
//    driving different devices do not wait for each other: each device has
//    its own lock and its own host read-back buffer;
//  * a launch needing more scratch than the array holds is rejected with an
//    error message, before anything runs;
//  * it runs the table-driven solve kernel (the network-specialized kernel
//    is compiled with NVRTC into memory the driver allocates): about 2.6x
//    slower than pfchem_react_batch on the 12-species network (918 vs 354 ms
//    per step at 2,097,152 cells);
//  * no cudaMalloc, cudaFree or other allocating routine is called.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/pfchem.h"
#include "pfchem_device.cuh"

namespace pfchem {
int flatten_network(const pfchem_network *w, const pfchem_options *o, DevNet &n, char *err, size_t errlen);
CellArgs cell_args(const pfchem_cells *cl, double dt);
int slots_blocks_per_sm(const DevNet &n, int block);
size_t slots_scratch_bytes(int grid);
cudaError_t launch_react_slots(const DevNet &n, const CellArgs &a, void *scratch, int grid, int block, int refill,
                               cudaStream_t st);
void sum_slots(const void *host_slots, int grid, unsigned long long *sum_iter, unsigned long long *alt,
               unsigned *max_iter, unsigned *bad);
}  // namespace pfchem

using namespace pfchem;

namespace {

// The scratch: 256 bytes of queue head, then 32-byte statistics slots, one
// per thread block of the persistent grid (at most 2040 blocks).
static __device__ __align__(256) unsigned char g_noalloc_scratch[PFCHEM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
// per device: a lock over that device's use of the state below, the device
// address of g_noalloc_scratch, and the host read-back of the slots
std::mutex g_mutex[kMaxDevices];
void *g_scratch_addr[kMaxDevices] = {};
unsigned char g_host_slots[kMaxDevices][PFCHEM_NOALLOC_SCRATCH_BYTES];

int err_out(char *err, size_t len, int code, const char *msg, const char *detail = nullptr) {
  if (err && len) {
    if (detail) snprintf(err, len, "%s: %s", msg, detail);
    else snprintf(err, len, "%s", msg);
  }
  return code;
}

}  // namespace

extern "C" int pfchem_react_batch_noalloc(const pfchem_network *net, const pfchem_options *opt, double dt,
                                          pfchem_cells *cells, void *stream, pfchem_stats *stats, char *err,
                                          size_t errlen) {
  if (!net || !opt || !cells) return err_out(err, errlen, -1, "null argument");
  if (!cells->on_device) return err_out(err, errlen, -1, "pfchem_react_batch_noalloc takes device pointers only");
  if (!(dt > 0.0)) return err_out(err, errlen, -1, "dt must be > 0");
  if (cells->ncells < 0) return err_out(err, errlen, -1, "ncells < 0");
  if (!cells->total || !cells->temperature || !cells->saturation || !cells->den_kg || !cells->porosity ||
      !cells->volume || !cells->pri_molal || !cells->ionic_strength)
    return err_out(err, errlen, -1, "a required per-cell array is null");
  DevNet n;
  char msg[512];
  if (flatten_network(net, opt, n, msg, sizeof(msg))) return err_out(err, errlen, -1, "invalid network", msg);
  if (n.Nm > 0 && (!cells->mnrl_volfrac || !cells->mnrl_area))
    return err_out(err, errlen, -1, "mnrl_volfrac/mnrl_area required");
  if (n.Nix + n.Nsr > 0 && !cells->total_sorb_eq) return err_out(err, errlen, -1, "total_sorb_eq required");
  if (n.Nix > 0 && !cells->eqionx_ref_cation_sorbed_conc)
    return err_out(err, errlen, -1, "eqionx_ref_cation_sorbed_conc required");
  if (n.Nsr > 0 && !cells->srfcplxrxn_free_site_conc)
    return err_out(err, errlen, -1, "srfcplxrxn_free_site_conc required");
  if (n.use_h2o && !cells->ln_act_h2o) return err_out(err, errlen, -1, "ln_act_h2o required");
  for (int r = 0; r < n.Nsr; ++r)
    if (n.srtype[r] == PFCHEM_ROCK_SURFACE && !cells->soil_particle_density)
      return err_out(err, errlen, -1, "soil_particle_density required for ROCK surfaces");

  if (stats) std::memset(stats, 0, sizeof(*stats));
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return err_out(err, errlen, -2, "cudaGetDevice", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return err_out(err, errlen, -1, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mutex[dev]);
  if (!g_scratch_addr[dev]) {
    // once per device, with the device current: the array's device address
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return err_out(err, errlen, -2, "cudaGetSymbolAddress", cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  void *scratch = g_scratch_addr[dev];
  if (cells->ncells == 0) return 0;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int block = 64;
  int bps = slots_blocks_per_sm(n, block);
  if (bps < 1) return err_out(err, errlen, -1, "the solve kernel does not fit on an SM for this network");
  // the persistent grid is sized to the scratch: at most as many resident
  // blocks per SM as there are statistics slots per SM
  const int max_slots = (int)((PFCHEM_NOALLOC_SCRATCH_BYTES - 256) / 32);
  if (sms > 0 && bps * sms > max_slots) bps = max_slots / sms > 0 ? max_slots / sms : 1;
  const int grid = sms * bps;
  const size_t need = slots_scratch_bytes(grid);
  if (need > PFCHEM_NOALLOC_SCRATCH_BYTES) {
    snprintf(msg, sizeof(msg), "the launch needs %zu bytes of scratch (%d blocks); the static scratch holds %d bytes",
             need, grid, PFCHEM_NOALLOC_SCRATCH_BYTES);
    return err_out(err, errlen, -1, msg);
  }
  cudaStream_t st = (cudaStream_t)stream;
  e = cudaMemsetAsync(scratch, 0, need, st);  // queue head and slots start at zero
  if (e != cudaSuccess) return err_out(err, errlen, -2, "cudaMemsetAsync", cudaGetErrorString(e));
  CellArgs a = cell_args(cells, dt);
  e = launch_react_slots(n, a, scratch, grid, block, 8, st);
  if (e != cudaSuccess) return err_out(err, errlen, -2, "solve launch", cudaGetErrorString(e));
  e = cudaMemcpyAsync(g_host_slots[dev], (char *)scratch + 256, need - 256, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return err_out(err, errlen, -2, "cudaMemcpyAsync", cudaGetErrorString(e));
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return err_out(err, errlen, -2, "cudaStreamSynchronize", cudaGetErrorString(e));
  unsigned long long sum_iter, alt;
  unsigned max_iter, bad;
  sum_slots(g_host_slots[dev], grid, &sum_iter, &alt, &max_iter, &bad);
  if (stats) {  // the fields not measured here (kernel_ms, lane_slots, drain_ms) stay 0
    stats->ncells = cells->ncells;
    stats->sum_iterations = (int64_t)sum_iter;
    stats->max_iterations = (int32_t)max_iter;
    stats->nonconverged = (int32_t)bad;
    stats->alt_guess_used = (int64_t)alt;
  }
  return (int)bad;
}
