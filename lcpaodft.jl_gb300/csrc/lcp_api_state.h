// Internal state of the C ABI objects (contexts, cells, orbital tables, jobs)
// shared by the translation units that orchestrate kernels.  Not part of the
// public interface.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "lcp_device.h"
#include "lcp_internal.h"

static inline lcp_status fail(lcp_status code, const std::string& msg) {
  lcp::set_error(msg);
  return code;
}

static inline lcp_status cuda_fail(cudaError_t e, const char* where) {
  return fail(e == cudaErrorMemoryAllocation ? LCP_ENOMEM : LCP_EDEVICE,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define API_CUDA(expr, where)                       \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) return cuda_fail(_e, where); \
  } while (0)

// Number of device allocations (cudaMalloc) made through DBuf since the
// library was loaded, across all contexts; read by lcp_device_alloc_count.
inline std::atomic<int64_t> g_device_allocs{0};
// Number of DBuf frees: with the allocations, any change of a device buffer
// a captured step graph could point into invalidates it (lcp_job_step).
inline std::atomic<int64_t> g_device_frees{0};

// Owning device buffer.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() {
    if (p) {
      cudaFree(p);
      g_device_frees.fetch_add(1, std::memory_order_relaxed);
    }
  }
  cudaError_t ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    if (p) {
      cudaFree(p);
      g_device_frees.fetch_add(1, std::memory_order_relaxed);
    }
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n ? n : 16);
    g_device_allocs.fetch_add(1, std::memory_order_relaxed);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) {
      cudaFree(p);
      g_device_frees.fetch_add(1, std::memory_order_relaxed);
    }
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

template <class T>
cudaError_t upload(DBuf& b, const std::vector<T>& v, cudaStream_t st) {
  cudaError_t e = b.ensure(v.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  e = cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

static inline int channels(int32_t spinpol) { return spinpol == LCP_SPIN_OFF ? 1 : (spinpol == LCP_SPIN_ON ? 2 : 4); }

struct lcp_ucell {
  lcp::UCell u;
};

// The hand-written FFT's plan of one grid shape: radices and roots of unity.
struct FftPlans {
  lcp::FftGeom geom{};
  DBuf roots;
  bool ok = false;
};

struct lcp_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  int32_t precision = LCP_PREC_FP64;
  int64_t launches = 0;
  std::map<std::tuple<int, int, int>, FftPlans> plans;
  // workspaces of the host-buffer entry points
  DBuf w_in[4], w_out[4], w_aux[4], w_real, w_spec, w_part, w_scal, w_a, w_b;
  DBuf w_dsym, w_status, w_hscratch, w_dscale, w_dtmp, w_vw, w_vscale, w_pfac;
  // second stream of the step: the xc pass runs there beside the FFT Poisson solve
  cudaStream_t aux = nullptr;
  // device address of the no-allocation density's fixed scratch array, looked
  // up by this context's first lcp_set_density_grid_noalloc call
  void* noalloc_scratch = nullptr;
  // failure-path tests only (lcp_ctx_set_fault_test): the split-BF16 density
  // kernel's poll limit (0: its default) and its stall switch
  uint32_t fault_poll = 0;
  int32_t xc_dfl = 0;  // drop-in GGA-PBE entry points in double-float (lcp_ctx_set_xc_arithmetic)
  int32_t step_graphs = 1;  // lcp_job_step replays a captured CUDA graph (lcp_ctx_set_step_graphs)
  int32_t fault_stall = 0;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // lcp_job_tc_kernel_ms: events around the tensor-core kernels of one step
  // (pairs [density spin 0..3][H channel 0..3]); null when not timing
  cudaEvent_t* tc_ev = nullptr;
  ~lcp_ctx() {
    cudaSetDevice(device);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (aux) cudaStreamDestroy(aux);
    if (own) cudaStreamDestroy(own);
  }
};

struct lcp_orbs {
  const lcp_ucell* ucell = nullptr;
  int device = 0;
  bool grad = false;
  int max_no = 0;
  // the pair items in two orbital classes, pairs of at most 16 orbitals per
  // atom first: each class's FP64/FP32 pair kernels use its own tile bound
  int64_t nitems_small = 0;
  int max_no_small = 0, max_no_large = 0;
  lcp::DevGeom geom{};
  lcp::DevPairs pairs{};
  // device arrays
  DBuf atv, gxyz, spe, sph_off, glist, clist, phi_off, numorbs;
  DBuf species, radial, buckets;
  DBuf phi, dphi[3], phi32;
  DBuf p_atom, p_jatom, p_boffp, p_boffq, p_self, p_lensoff, p_g1, p_g2, it_pair, it_start, it_count;
  DBuf f_off, f_code;  // per atom, its work-item halves (item * 2 + orientation) for the force term
  int64_t table_elems = 0;
  // brick tiling and split-BF16 tables of the tensor-core path (built on first use)
  bool bricks_ready = false;
  int32_t brick_shape[3] = {0, 0, 0};  // requested brick shape, {0,0,0}: the predicted best
  bool phi_released = false;           // FP64/FP32 tables freed (split-BF16 tables only)
  lcp::Bricks bricks;
  lcp::TcBrickGeom bgeom{};
  DBuf b_code, b_imgoff, b_imgblk, b_taboff, b_tabpair, b_tab, b_tabslot, b_slotbase, b_redoff, b_redslot;
  DBuf b_subpair, b_subchunks, b_sbfold, b_sbchunks;  // sub-pairs and H sub-blocks (orbital chunks)
  DBuf o_atom, o_jatom, o_boff, o_partner;  // ordered pair list
  DBuf b_scale, b_tmp;                       // fixed-point scale of the tables: [S_phi, 1/S_phi]
  double phi_scale = 1.0;
  // device times of the last tabulation and split-table build (ms)
  float tab_ms = 0.f, split_ms = 0.f;
};

struct lcp_job {
  const lcp_ucell* ucell = nullptr;
  const lcp_orbs* orbs = nullptr;
  int32_t spinpol = LCP_SPIN_OFF, xc = LCP_XC_LDA;
  int nspin = 1;
  int64_t nn = 0, hsize = 0;
  double recvecs[9] = {};
  DBuf dm[4], rho[4], hks[4], vpot[4];
  DBuf aden, pcc, vna, dvh, real, spec, part, scal;
  DBuf pfac;  // Poisson factors of the half spectrum, tabulated at creation
  DBuf dcoef, dexc;  // GGA_PBE: stencil weights [3][27] and dE/d(grad rho) [spin][xyz][nn]
  bool has_aden = false, has_pcc = false, has_vna = false;
  FftPlans* plans = nullptr;
  // lcp_job_step's CUDA graphs, one per context that steps the job: the
  // step's launches captured once and replayed by one graph launch while
  // nothing they depend on changed (the signature: the context's stream and
  // options, and the device allocation and free counters).
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    int64_t sig[8] = {};    // signature the graph was captured under
    int64_t prev[8] = {};   // signature after the last step run without a graph
    int64_t launches = 0;   // kernels of the captured step
    bool have_prev = false, off = false;
  };
  std::map<const lcp_ctx*, StepGraph> graphs;
  lcp_job() = default;
  lcp_job(const lcp_job&) = delete;
  lcp_job& operator=(const lcp_job&) = delete;
  ~lcp_job() {
    for (auto& kv : graphs)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  }
};


// helpers of lcp_api.cu used by the other orchestration files
lcp_status get_plans(lcp_ctx* ctx, const int32_t* ng, FftPlans** out);
lcp_status make_fft_plan(const int32_t* ng, FftPlans* p);
lcp_status check_ctx(lcp_ctx* ctx);
lcp_status check_pair(const lcp_ucell* ucell, const lcp_orbs* orbs);
lcp_status ensure_bricks(lcp_ctx* ctx, lcp_orbs* o);
lcp_status device_status(lcp_ctx* ctx);
lcp_status density_device(lcp_ctx* ctx, const lcp_orbs* orbs, int nspin, const double* const* dm, double* const* rho,
                          int64_t nn);
lcp_status hamiltonian_device(lcp_ctx* ctx, const lcp_orbs* orbs, int nch, const double* const* vpot,
                              double* const* hks, int64_t hsize);
lcp::GridCell job_grid_cell(lcp_job* job);

int64_t job_footprint_estimate(lcp_job* job, int32_t precision);

// batches re-assembled over changing sets of jobs (lcp_batch.cu), for the serving engine
lcp_batch* batch_new(int device);
lcp_status batch_assemble(lcp_ctx* ctx, lcp_batch* b, int32_t njobs, lcp_job* const* jobs, int64_t scratch_bytes);
lcp_status batch_record(lcp_batch* b, cudaStream_t st);
lcp_status batch_status(lcp_batch* b, cudaStream_t st);
