// C ABI of the lcpgrid library: argument checking, device memory, and the
// orchestration of the kernels.  Declarations and conventions: lcpgrid.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "lcp_api_state.h"

using lcp::DevGeom;
using lcp::DevPairs;
using lcp::DevSpecies;

namespace lcp {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }
}  // namespace lcp

// Radices and roots of unity of a grid shape for the FFT Poisson solve.
lcp_status make_fft_plan(const int32_t* ng, FftPlans* p) {
  if (!lcp::fft_supported(ng))
    return fail(LCP_ENOTSUP, "the FFT Poisson solve takes grid dimensions of 1 to " +
                                 std::to_string(lcp::kFftMaxN) + " points");
  std::vector<double> r64, a64;
  std::vector<float> r32, a32;
  size_t o64[3], o32[3];
  for (int d = 0; d < 3; ++d) {
    p->geom.n[d] = ng[d];
    p->geom.nfac[d] = lcp::fft_factor(ng[d], p->geom.fac[d]);
    lcp::fft_roots(ng[d], r64, r32);
    o64[d] = a64.size();
    o32[d] = a32.size();
    a64.insert(a64.end(), r64.begin(), r64.end());
    a32.insert(a32.end(), r32.begin(), r32.end());
  }
  const size_t b64 = a64.size() * sizeof(double);
  API_CUDA(p->roots.ensure(b64 + a32.size() * sizeof(float)), "FFT roots alloc");
  API_CUDA(cudaMemcpy(p->roots.p, a64.data(), b64, cudaMemcpyHostToDevice), "FFT roots upload");
  API_CUDA(cudaMemcpy(static_cast<char*>(p->roots.p) + b64, a32.data(), a32.size() * sizeof(float),
                      cudaMemcpyHostToDevice),
           "FFT roots upload");
  for (int d = 0; d < 3; ++d) {
    p->geom.roots64[d] = p->roots.as<double>() + o64[d];
    p->geom.roots32[d] = reinterpret_cast<float*>(static_cast<char*>(p->roots.p) + b64) + o32[d];
  }
  p->ok = true;
  return LCP_OK;
}

lcp_status get_plans(lcp_ctx* ctx, const int32_t* ng, FftPlans** out) {
  auto key = std::make_tuple((int)ng[0], (int)ng[1], (int)ng[2]);
  auto it = ctx->plans.find(key);
  if (it == ctx->plans.end()) {
    it = ctx->plans.emplace(std::piecewise_construct, std::forward_as_tuple(key), std::forward_as_tuple()).first;
    lcp_status s = make_fft_plan(ng, &it->second);
    if (s) {
      ctx->plans.erase(it);
      return s;
    }
  }
  *out = &it->second;
  return LCP_OK;
}

// dvh = Poisson(real source already in `real`), with the factors tabulated
// into the context's workspace; spec is scratch.
lcp_status poisson_device(lcp_ctx* ctx, FftPlans* pl, const int32_t* ng, const double* recvecs, double* real,
                          void* spec, double* dvh) {
  const int64_t nspec = (int64_t)ng[0] * ng[1] * (ng[2] / 2 + 1);
  API_CUDA(ctx->w_pfac.ensure(nspec * sizeof(double)), "alloc");
  API_CUDA(lcp::launch_poisson_table(ng, recvecs, ctx->w_pfac.as<double>(), ctx->stream), "poisson table");
  lcp::GridCell c{};
  for (int d = 0; d < 3; ++d) c.ng[d] = ng[d];
  c.nn = (int64_t)ng[0] * ng[1] * ng[2];
  c.real = real;
  c.spec = spec;
  c.pfac = ctx->w_pfac.as<double>();
  c.dvh = dvh;
  API_CUDA(lcp::launch_poisson_fft(pl->geom, ctx->precision == LCP_PREC_FP64, -1, c, nullptr, 1, ctx->stream),
           "poisson fft");
  ctx->launches += 6;
  return LCP_OK;
}

lcp_status check_ctx(lcp_ctx* ctx) {
  if (!ctx) return fail(LCP_EINVAL, "context is NULL");
  API_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  return LCP_OK;
}

lcp_status check_pair(const lcp_ucell* ucell, const lcp_orbs* orbs) {
  if (!ucell || !orbs) return fail(LCP_EINVAL, "ucell/orbs is NULL");
  if (orbs->ucell != ucell) return fail(LCP_EINVAL, "Orbs_Grid was tabulated for a different UCell");
  return LCP_OK;
}

lcp_status ensure_phi32(lcp_ctx* ctx, lcp_orbs* o) {
  if (o->phi32.p) return LCP_OK;
  if (o->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released");
  API_CUDA(o->phi32.ensure(o->table_elems * sizeof(float)), "phi32 alloc");
  API_CUDA(lcp::launch_convert_f32(o->phi.as<double>(), o->phi32.as<float>(), o->table_elems, ctx->stream),
           "convert_f32");
  ctx->launches++;
  return LCP_OK;
}

// Brick tiling, split-BF16 orbital tables and the ordered pair list of the
// tensor-core path, built once per tabulation.
lcp_status ensure_bricks(lcp_ctx* ctx, lcp_orbs* o) {
  if (o->bricks_ready) return LCP_OK;
  if (o->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released");
  const lcp::UCell& u = o->ucell->u;
  lcp::Bricks& b = o->bricks;
  std::string err = lcp::build_bricks(u, b, o->brick_shape[0] > 0 ? o->brick_shape : nullptr);
  if (!err.empty()) return fail(LCP_EINVAL, err);
  if (b.max_images > lcp::kMaxBrickImages)
    return fail(LCP_ENOTSUP, "a grid brick is touched by " + std::to_string(b.max_images) +
                                 " atom images (16-orbital chunks); the tensor-core path supports " +
                                 std::to_string(lcp::kMaxBrickImages));
  cudaStream_t st = ctx->stream;
  API_CUDA(upload(o->b_code, b.point_code, st), "upload");
  API_CUDA(upload(o->b_imgoff, b.img_off, st), "upload");
  API_CUDA(upload(o->b_imgblk, b.img_block, st), "upload");
  API_CUDA(upload(o->b_taboff, b.tab_off, st), "upload");
  API_CUDA(upload(o->b_tabpair, b.tab_pair, st), "upload");
  API_CUDA(upload(o->b_tabslot, b.tab_slot, st), "upload");
  API_CUDA(upload(o->b_slotbase, b.slot_base, st), "upload");
  API_CUDA(upload(o->b_redoff, b.red_off, st), "upload");
  API_CUDA(upload(o->b_redslot, b.red_slot, st), "upload");
  API_CUDA(upload(o->b_subpair, b.sub_pair, st), "upload");
  API_CUDA(upload(o->b_subchunks, b.sub_chunks, st), "upload");
  API_CUDA(upload(o->b_sbfold, b.sb_fold, st), "upload");
  API_CUDA(upload(o->b_sbchunks, b.sb_chunks, st), "upload");
  std::vector<int64_t> boff(u.block_off.begin(), u.block_off.end());
  API_CUDA(upload(o->o_atom, u.pair_atom, st), "upload");
  API_CUDA(upload(o->o_jatom, u.pair_jatom, st), "upload");
  API_CUDA(upload(o->o_boff, boff, st), "upload");
  API_CUDA(upload(o->o_partner, u.partner, st), "upload");
  API_CUDA(o->b_tab.ensure((size_t)std::max<int64_t>(b.nblocks, 1) * 6144 * 2), "brick table alloc");
  API_CUDA(o->b_scale.ensure(2 * sizeof(double)), "alloc");
  API_CUDA(o->b_tmp.ensure(sizeof(unsigned long long)), "alloc");
  // the first block of every atom image: images take ceil(NO / 16) consecutive blocks
  std::vector<int32_t> first;
  for (int64_t blk = 0; blk < b.nblocks;) {
    first.push_back((int32_t)blk);
    blk += (u.numorbs[b.block_atom[blk]] + 15) / 16;
  }
  DBuf d_first, d_batom, d_slots;
  API_CUDA(upload(d_first, first, st), "upload");
  API_CUDA(upload(d_batom, b.block_atom, st), "upload");
  API_CUDA(d_slots.ensure((size_t)std::max<int64_t>(b.nblocks, 1) * 128 * sizeof(int32_t)), "table slots alloc");
  // device time of the build (scale, slot map, tables), without the host work above
  cudaEvent_t te[2];
  API_CUDA(cudaEventCreate(&te[0]), "event");
  API_CUDA(cudaEventCreate(&te[1]), "event");
  API_CUDA(cudaEventRecord(te[0], st), "event");
  API_CUDA(lcp::launch_absmax_scale(o->phi.as<double>(), o->table_elems, 1.0, o->b_tmp.as<unsigned long long>(),
                                    o->b_scale.as<double>(), st),
           "table scale");
  API_CUDA(lcp::launch_brick_table(o->phi.as<double>(), o->geom.phi_off, o->geom.numorbs, o->geom.sph_off,
                                   o->b_code.as<int32_t>(), (int64_t)b.point_code.size(), d_batom.as<int32_t>(),
                                   d_first.as<int32_t>(), (int64_t)first.size(), d_slots.as<int32_t>(),
                                   o->b_scale.as<double>(), o->b_tab.as<__nv_bfloat16>(), b.nblocks, st),
           "brick table");
  API_CUDA(cudaEventRecord(te[1], st), "event");
  API_CUDA(cudaStreamSynchronize(st), "brick table");  // before the scratch above is freed
  cudaEventElapsedTime(&o->split_ms, te[0], te[1]);
  cudaEventDestroy(te[0]);
  cudaEventDestroy(te[1]);
  ctx->launches += 4;
  API_CUDA(cudaMemcpyAsync(&o->phi_scale, o->b_scale.p, sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  lcp::TcBrickGeom& g = o->bgeom;
  g.nbricks = b.nbricks;
  g.nblocks = b.nblocks;
  for (int d = 0; d < 3; ++d) {
    g.bdim[d] = b.bdim[d];
    g.nb[d] = b.nb[d];
    g.ngrid[d] = u.ngrid[d];
  }
  g.npts = b.npts;
  g.max_images = b.max_images;
  g.img_off = o->b_imgoff.as<int64_t>();
  g.img_block = o->b_imgblk.as<int32_t>();
  g.tab_off = o->b_taboff.as<int64_t>();
  g.tab_pair = o->b_tabpair.as<int32_t>();
  API_CUDA(cudaStreamSynchronize(st), "bricks");
  o->bricks_ready = true;
  return LCP_OK;
}

namespace {
void drop_bricks(lcp_orbs* o) {
  o->bricks_ready = false;
  o->bricks = lcp::Bricks();
  for (DBuf* d : {&o->b_code, &o->b_imgoff, &o->b_imgblk, &o->b_taboff, &o->b_tabpair, &o->b_tab, &o->b_tabslot,
                  &o->b_slotbase, &o->b_redoff, &o->b_redslot, &o->b_subpair, &o->b_subchunks, &o->b_sbfold,
                  &o->b_sbchunks})
    d->release();
}

__global__ void fill_kernel(double* x, int64_t n, double v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}
}  // namespace

lcp_status density_tc_device(lcp_ctx* ctx, const lcp_orbs* orbs_c, int nspin, const double* const* dm,
                             double* const* rho) {
  lcp_orbs* o = const_cast<lcp_orbs*>(orbs_c);
  lcp_status s = ensure_bricks(ctx, o);
  if (s) return s;
  const lcp::UCell& u = o->ucell->u;
  const int64_t nsub = o->bricks.nsub;
  API_CUDA(ctx->w_dsym.ensure((size_t)(nsub + 1) * 768 * 2), "dsym alloc");
  API_CUDA(ctx->w_dscale.ensure(2 * sizeof(double)), "alloc");
  API_CUDA(ctx->w_dtmp.ensure(sizeof(unsigned long long)), "alloc");
  for (int c = 0; c < nspin; ++c) {
    // |D + D'^T| <= 2 max|D|: the fixed-point scale of the symmetrised blocks
    API_CUDA(lcp::launch_absmax_scale(dm[c], u.total_hsize, 2.0, ctx->w_dtmp.as<unsigned long long>(),
                                      ctx->w_dscale.as<double>(), ctx->stream),
             "dm scale");
    API_CUDA(lcp::launch_dsym(nsub, o->b_subpair.as<int32_t>(), o->b_subchunks.as<int32_t>(), o->o_atom.as<int32_t>(),
                              o->o_jatom.as<int32_t>(), o->o_boff.as<int64_t>(), o->o_partner.as<int32_t>(),
                              o->geom.numorbs, dm[c], ctx->w_dscale.as<double>(),
                              ctx->w_dsym.as<__nv_bfloat16>(), ctx->stream),
             "dsym");
    if (ctx->tc_ev) API_CUDA(cudaEventRecord(ctx->tc_ev[2 * c], ctx->stream), "event");
    API_CUDA(lcp::launch_density_tc(o->bgeom, o->b_tab.as<__nv_bfloat16>(), o->phi_scale,
                                    ctx->w_dsym.as<__nv_bfloat16>(), ctx->w_dscale.as<double>(), (int)nsub, rho[c],
                                    ctx->w_status.as<int>(), ctx->stream, ctx->fault_poll, ctx->fault_stall),
             "density_tc");
    if (ctx->tc_ev) API_CUDA(cudaEventRecord(ctx->tc_ev[2 * c + 1], ctx->stream), "event");
    ctx->launches += 4;
  }
  return LCP_OK;
}

// Runs launch(items, max orbitals, first item) on each orbital class of the
// pair items (see lcp_orbs::nitems_small); returns the number of launches.
template <class F>
cudaError_t for_item_classes(const lcp_orbs* o, int* launches, F launch) {
  const lcp::DevPairs& pr = o->pairs;
  *launches = 0;
  if (o->nitems_small > 0) {
    lcp::DevPairs a = pr;
    a.nitems = o->nitems_small;
    LCP_CUDA_TRY(launch(a, o->max_no_small, (int64_t)0));
    ++*launches;
  }
  const int64_t nl = pr.nitems - o->nitems_small;
  if (nl > 0) {
    lcp::DevPairs b = pr;
    b.nitems = nl;
    b.item_pair += o->nitems_small;
    b.item_start += o->nitems_small;
    b.item_count += o->nitems_small;
    LCP_CUDA_TRY(launch(b, o->max_no_large, o->nitems_small));
    ++*launches;
  }
  return cudaSuccess;
}

lcp_status density_device(lcp_ctx* ctx, const lcp_orbs* orbs, int nspin, const double* const* dm, double* const* rho,
                          int64_t nn) {
  int prec = ctx->precision;
  if (prec == LCP_PREC_BF16X3) return density_tc_device(ctx, orbs, nspin, dm, rho);
  if (orbs->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released (split-BF16 only)");
  for (int s = 0; s < nspin; ++s) API_CUDA(cudaMemsetAsync(rho[s], 0, nn * sizeof(double), ctx->stream), "memset");
  if (prec == LCP_PREC_FP32) {
    lcp_status s = ensure_phi32(ctx, const_cast<lcp_orbs*>(orbs));
    if (s != LCP_OK) return s;
  }
  int nl = 0;
  API_CUDA(for_item_classes(orbs, &nl,
                            [&](const lcp::DevPairs& pr, int max_no, int64_t) {
                              return lcp::launch_density_pairs(prec, orbs->geom, pr, nspin, orbs->phi.as<double>(),
                                                               orbs->phi32.as<float>(), dm, rho, max_no, ctx->stream);
                            }),
           "density kernel");
  ctx->launches += nl;
  return LCP_OK;
}

// Error word written by kernels whose bounded waits gave up; read and cleared.
lcp_status device_status(lcp_ctx* ctx) {
  int st = 0;
  API_CUDA(cudaMemcpy(&st, ctx->w_status.p, sizeof(int), cudaMemcpyDeviceToHost), "status");
  if (st) {
    cudaMemset(ctx->w_status.p, 0, sizeof(int));
    return fail(st, "a device wait timed out (tensor-core completion)");
  }
  return LCP_OK;
}

lcp_status hamiltonian_tc_device(lcp_ctx* ctx, const lcp_orbs* orbs_c, int nch, const double* const* vpot,
                                 double* const* hks) {
  lcp_orbs* o = const_cast<lcp_orbs*>(orbs_c);
  lcp_status s = ensure_bricks(ctx, o);
  if (s) return s;
  const lcp::UCell& u = o->ucell->u;
  const int64_t nslots = o->bricks.slot_base.back();
  API_CUDA(ctx->w_hscratch.ensure((size_t)std::max<int64_t>(nslots, 1) * 256 * sizeof(float)), "H scratch alloc");
  const size_t nb = (size_t)std::max<int64_t>(o->bgeom.nbricks, 1);
  API_CUDA(ctx->w_vw.ensure(nb * 128 * sizeof(float2)), "V weight alloc");
  API_CUDA(ctx->w_vscale.ensure(nb * sizeof(float)), "V scale alloc");
  for (int c = 0; c < nch; ++c) {
    API_CUDA(lcp::launch_hamiltonian_tc(o->bgeom, o->b_tabslot.as<int32_t>(), o->b_slotbase.as<int64_t>(),
                                        o->b_tab.as<__nv_bfloat16>(), o->phi_scale, vpot[c], ctx->w_vw.as<float2>(),
                                        ctx->w_vscale.as<float>(), ctx->w_hscratch.as<float>(),
                                        ctx->w_status.as<int>(), ctx->stream,
                                        ctx->tc_ev ? ctx->tc_ev[8 + 2 * c] : nullptr,
                                        ctx->tc_ev ? ctx->tc_ev[8 + 2 * c + 1] : nullptr),
             "hamiltonian_tc");
    API_CUDA(lcp::launch_h_reduce((int64_t)o->bricks.sb_fold.size(), o->b_redoff.as<int64_t>(),
                                  o->b_redslot.as<int64_t>(), o->b_sbfold.as<int32_t>(), o->b_sbchunks.as<int32_t>(),
                                  ctx->w_hscratch.as<float>(), o->pairs, o->geom.numorbs, u.gridvol, hks[c],
                                  ctx->stream),
             "h_reduce");
    ctx->launches += 3;
  }
  return LCP_OK;
}

lcp_status hamiltonian_device(lcp_ctx* ctx, const lcp_orbs* orbs, int nch, const double* const* vpot,
                              double* const* hks, int64_t hsize) {
  int prec = ctx->precision;
  if (prec == LCP_PREC_BF16X3) return hamiltonian_tc_device(ctx, orbs, nch, vpot, hks);
  if (orbs->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released (split-BF16 only)");
  for (int c = 0; c < nch; ++c) API_CUDA(cudaMemsetAsync(hks[c], 0, hsize * sizeof(double), ctx->stream), "memset");
  if (prec == LCP_PREC_FP32) {
    lcp_status s = ensure_phi32(ctx, const_cast<lcp_orbs*>(orbs));
    if (s != LCP_OK) return s;
  }
  int nl = 0;
  API_CUDA(for_item_classes(orbs, &nl,
                            [&](const lcp::DevPairs& pr, int max_no, int64_t) {
                              return lcp::launch_hamiltonian_pairs(prec, orbs->geom, pr, nch, orbs->phi.as<double>(),
                                                                   orbs->phi32.as<float>(), vpot, hks, max_no,
                                                                   ctx->stream);
                            }),
           "hamiltonian kernel");
  ctx->launches += nl;
  return LCP_OK;
}



// The job's cell as a grid-step pass sees it (its own buffers).
lcp::GridCell job_grid_cell(lcp_job* job) {
  const lcp::UCell& u = job->ucell->u;
  lcp::GridCell c{};
  for (int d = 0; d < 3; ++d) c.ng[d] = u.ngrid[d];
  c.nn = job->nn;
  c.hsize = job->hsize;
  for (int d = 0; d < 9; ++d) c.rv[d] = job->recvecs[d];
  c.gridvol = u.gridvol;
  c.aden = job->has_aden ? job->aden.as<double>() : nullptr;
  c.pcc = job->has_pcc ? job->pcc.as<double>() : nullptr;
  c.vna = job->has_vna ? job->vna.as<double>() : nullptr;
  for (int s = 0; s < job->nspin && s < 4; ++s) {
    c.rho[s] = job->rho[s].as<double>();
    c.vpot[s] = job->vpot[s].as<double>();
    c.dm[s] = job->dm[s].as<double>();
    c.hks[s] = job->hks[s].as<double>();
  }
  c.real = job->real.as<double>();
  c.spec = job->spec.p;
  c.pfac = job->pfac.as<double>();
  c.dvh = job->dvh.as<double>();
  c.part = job->part.as<double>();
  c.sums = job->scal.as<double>();
  if (job->xc == LCP_XC_GGA_PBE) {
    c.dcoef = job->dcoef.as<double>();
    c.dexc = job->dexc.as<double>();
  }
  return c;
}

// gLatvecs: Latvecs rows / Ngrid (src/Energy.jl:676-679)
static void grid_vectors(const double* lat, const int32_t* ngrid, double gtv[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int d = 0; d < 3; ++d) gtv[i][d] = lat[i * 3 + d] / ngrid[i];
}

extern "C" {

const char* lcp_last_error(void) { return lcp::last_error_cstr(); }
const char* lcp_version(void) { return "lcpgrid 0.1 (sm_103a)"; }

// ---------------------------------------------------------------- geometry

lcp_status lcp_ucell_create(int32_t nspin, const double* latvecs, int32_t natom, const int32_t* atom2spe,
                            const double* gxyz, const double* atoms_cut1, const int32_t* ngrid,
                            const double* grid_origin, const int32_t* total_numorbs, lcp_ucell** out) {
  if (!out || !latvecs || !atom2spe || !gxyz || !atoms_cut1 || !ngrid) return fail(LCP_EINVAL, "NULL argument");
  *out = nullptr;
  std::unique_ptr<lcp_ucell> u(new (std::nothrow) lcp_ucell());
  if (!u) return fail(LCP_ENOMEM, "out of host memory");
  try {
    std::string err = lcp::build_ucell(u->u, nspin, latvecs, natom, atom2spe, gxyz, atoms_cut1, ngrid, grid_origin,
                                       total_numorbs);
    if (!err.empty()) return fail(LCP_EINVAL, err);
  } catch (const std::bad_alloc&) {
    return fail(LCP_ENOMEM, "out of host memory building UCell");
  }
  *out = u.release();
  return LCP_OK;
}

void lcp_ucell_destroy(lcp_ucell* ucell) { delete ucell; }

lcp_status lcp_ucell_get_info(const lcp_ucell* ucell, lcp_ucell_info* info) {
  if (!ucell || !info) return fail(LCP_EINVAL, "NULL argument");
  const lcp::UCell& u = ucell->u;
  info->cpycell = u.cpycell;
  info->natom = u.natom;
  info->nloop = u.nloop;
  info->ncell = u.ncell;
  for (int d = 0; d < 3; ++d) info->ngrid[d] = u.ngrid[d];
  info->max_numorbs = u.max_numorbs();
  info->total_hsize = u.total_hsize;
  info->sum_gridn = u.sphere_off.empty() ? 0 : u.sphere_off.back();
  int64_t so = 0;
  for (auto v : u.numolg) so += v;
  info->sum_numolg = so;
  info->n_unique = (int64_t)u.uniq_pair.size();
  info->gridvol = u.gridvol;
  return LCP_OK;
}

lcp_status lcp_ucell_get_int(const lcp_ucell* ucell, int32_t field, int64_t index, int32_t* dst, int64_t count) {
  if (!ucell || (!dst && count > 0)) return fail(LCP_EINVAL, "NULL argument");
  const lcp::UCell& u = ucell->u;
  std::vector<int32_t> tmp;
  const int32_t* src = nullptr;
  int64_t n = 0;
  auto need_atom = [&]() { return index >= 0 && index < u.natom; };
  auto need_pair = [&]() { return index >= 0 && index < u.nloop; };
  switch (field) {
    case LCP_F_FNAN: src = u.fnan.data(); n = u.natom; break;
    case LCP_F_NATN:
      if (!need_atom()) return fail(LCP_EINVAL, "atom index out of range");
      src = u.natn[index].data(); n = (int64_t)u.natn[index].size(); break;
    case LCP_F_NCN:
      if (!need_atom()) return fail(LCP_EINVAL, "atom index out of range");
      src = u.ncn[index].data(); n = (int64_t)u.ncn[index].size(); break;
    case LCP_F_GRIDN_ATOM:
      for (int a = 0; a < u.natom; ++a) tmp.push_back((int32_t)(u.sphere_off[a + 1] - u.sphere_off[a]));
      src = tmp.data(); n = u.natom; break;
    case LCP_F_GRIDLIST:
    case LCP_F_CELLLIST:
      if (!need_atom()) return fail(LCP_EINVAL, "atom index out of range");
      src = (field == LCP_F_GRIDLIST ? u.glist.data() : u.clist.data()) + u.sphere_off[index];
      n = u.sphere_off[index + 1] - u.sphere_off[index]; break;
    case LCP_F_PAIR_ATOM:
    case LCP_F_PAIR_NATN:
      for (int p = 0; p < u.nloop; ++p) tmp.push_back((field == LCP_F_PAIR_ATOM ? u.pair_atom[p] : u.pair_jatom[p]) + 1);
      src = tmp.data(); n = u.nloop; break;
    case LCP_F_PAIR_NCN: src = u.pair_cell.data(); n = u.nloop; break;
    case LCP_F_NUMOLG:
      for (int p = 0; p < u.nloop; ++p) tmp.push_back((int32_t)u.numolg[p]);
      src = tmp.data(); n = u.nloop; break;
    case LCP_F_GLIST1:
    case LCP_F_GLIST2: {
      if (!need_pair()) return fail(LCP_EINVAL, "pair index out of range");
      std::vector<int32_t> g1, g2;
      lcp::pair_overlap(u, (int32_t)index, g1, g2);
      tmp = field == LCP_F_GLIST1 ? g1 : g2;
      src = tmp.data(); n = (int64_t)tmp.size(); break;
    }
    case LCP_F_ATV_IJK: src = u.atv_ijk.data(); n = (int64_t)u.atv_ijk.size(); break;
    default: return fail(LCP_EINVAL, "unknown field");
  }
  if (count != n) return fail(LCP_EINVAL, "count does not match the field length " + std::to_string(n));
  if (n) std::memcpy(dst, src, n * sizeof(int32_t));
  return LCP_OK;
}

lcp_status lcp_ucell_get_bricks(const lcp_ucell* ucell, int64_t* info) {
  if (!ucell || !info) return fail(LCP_EINVAL, "NULL argument");
  lcp::Bricks b;
  std::string err = lcp::build_bricks(ucell->u, b);
  if (!err.empty()) return fail(LCP_EINVAL, err);
  for (int d = 0; d < 3; ++d) {
    info[d] = b.bdim[d];
    info[3 + d] = b.nb[d];
  }
  info[6] = b.npts;
  info[7] = b.nbricks;
  info[8] = b.nblocks;
  info[9] = b.max_images;
  int64_t paired = 0;
  for (auto v : b.tab_pair) paired += v >= 0;
  info[10] = (int64_t)b.img_block.size();
  info[11] = paired;
  info[12] = b.slot_base.empty() ? 0 : b.slot_base.back();
  info[13] = b.nsub;
  return LCP_OK;
}

lcp_status lcp_brick_shape_candidates(const lcp_ucell* ucell, int32_t max, int32_t* shapes, double* cost,
                                      int32_t* n) {
  if (!ucell || !shapes || !n || max < 0) return fail(LCP_EINVAL, "NULL argument");
  std::vector<double> c;
  auto cand = lcp::brick_shape_candidates(ucell->u, &c);
  const int k = (int)std::min<size_t>(cand.size(), (size_t)max);
  for (int i = 0; i < k; ++i) {
    for (int d = 0; d < 3; ++d) shapes[3 * i + d] = cand[i][d];
    if (cost) cost[i] = c[i];
  }
  *n = k;
  return LCP_OK;
}

lcp_status lcp_ucell_get_atv(const lcp_ucell* ucell, double* dst) {
  if (!ucell || !dst) return fail(LCP_EINVAL, "NULL argument");
  std::memcpy(dst, ucell->u.atv.data(), ucell->u.atv.size() * sizeof(double));
  return LCP_OK;
}

lcp_status lcp_calc_ngrid(double ecut, const double* L, int32_t* ngrid_out) {
  if (!L || !ngrid_out) return fail(LCP_EINVAL, "NULL argument");
  if (ecut < 0.0) return fail(LCP_EINVAL, "please check Ecut.");
  // src/utils/Calc_Ngrid.jl:1-76
  auto cross_norm = [&](int a, int b) {
    double x = L[a * 3 + 1] * L[b * 3 + 2] - L[a * 3 + 2] * L[b * 3 + 1];
    double y = L[a * 3 + 2] * L[b * 3 + 0] - L[a * 3 + 0] * L[b * 3 + 2];
    double z = L[a * 3 + 0] * L[b * 3 + 1] - L[a * 3 + 1] * L[b * 3 + 0];
    return std::sqrt(x * x + y * y + z * z);
  };
  double det = L[0] * (L[4] * L[8] - L[5] * L[7]) - L[1] * (L[3] * L[8] - L[5] * L[6]) + L[2] * (L[3] * L[7] - L[4] * L[6]);
  double temp = std::fabs(det) / 3.14159265358979323846 * std::sqrt(ecut);
  double ns[3] = {temp / cross_norm(1, 2), temp / cross_norm(2, 0), temp / cross_norm(0, 1)};
  for (int d = 0; d < 3; ++d) {
    double lgn = std::log(ns[d]);
    double best = 1e10;
    int bp = 0, bq = 0, br = 0, bs = 0;
    const double l2 = std::log(2.0), l3 = std::log(3.0), l5 = std::log(5.0), l7 = std::log(7.0);
    for (int p = 0; p <= (int)std::ceil(lgn / l2); ++p)
      for (int q = 0; q <= (int)std::ceil((lgn - p * l2) / l3); ++q)
        for (int r = 0; r <= (int)std::ceil((lgn - p * l2 - q * l3) / l5); ++r)
          for (int s = 0; s <= (int)std::ceil((lgn - p * l2 - q * l3 - r * l5) / l7); ++s) {
            double lg = p * l2 + q * l3 + r * l5 + s * l7;
            if (std::fabs(lg - lgn) < best) {
              best = std::fabs(lg - lgn);
              bp = p; bq = q; br = r; bs = s;
            }
          }
    int k = 1;
    for (int i = 0; i < bp; ++i) k *= 2;
    for (int i = 0; i < bq; ++i) k *= 3;
    for (int i = 0; i < br; ++i) k *= 5;
    for (int i = 0; i < bs; ++i) k *= 7;
    ngrid_out[d] = k;
  }
  return LCP_OK;
}

// ---------------------------------------------------------------- context

lcp_status lcp_ctx_create(int32_t device, lcp_ctx** out) {
  if (!out) return fail(LCP_EINVAL, "NULL argument");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(LCP_EDEVICE, "no CUDA device available");
  if (device < 0 || device >= n) return fail(LCP_EINVAL, "device index out of range");
  API_CUDA(cudaSetDevice(device), "cudaSetDevice");
  std::unique_ptr<lcp_ctx> c(new lcp_ctx());
  c->device = device;
  API_CUDA(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking), "cudaStreamCreate");
  c->stream = c->own;
  API_CUDA(c->w_status.ensure(sizeof(int)), "status alloc");
  API_CUDA(cudaMemset(c->w_status.p, 0, sizeof(int)), "memset");
  *out = c.release();
  return LCP_OK;
}

void lcp_ctx_destroy(lcp_ctx* ctx) { delete ctx; }

lcp_status lcp_ctx_set_stream(lcp_ctx* ctx, void* stream) {
  if (!ctx) return fail(LCP_EINVAL, "context is NULL");
  ctx->stream = stream ? reinterpret_cast<cudaStream_t>(stream) : ctx->own;
  return LCP_OK;
}

lcp_status lcp_ctx_set_precision(lcp_ctx* ctx, int32_t precision) {
  if (!ctx) return fail(LCP_EINVAL, "context is NULL");
  if (precision < LCP_PREC_FP64 || precision > LCP_PREC_BF16X3) return fail(LCP_EINVAL, "unknown precision");
  ctx->precision = precision;
  return LCP_OK;
}

lcp_status lcp_ctx_synchronize(lcp_ctx* ctx) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  API_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return LCP_OK;
}

int64_t lcp_ctx_launch_count(const lcp_ctx* ctx) { return ctx ? ctx->launches : -1; }

// ---------------------------------------------------------------- orbitals

lcp_status lcp_set_orbitals_grid(lcp_ctx* ctx, const lcp_ucell* ucell, int32_t nspecies, const lcp_pao* paos,
                                 int32_t with_grad, lcp_orbs** out) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!ucell || !paos || !out || nspecies <= 0) return fail(LCP_EINVAL, "NULL argument");
  *out = nullptr;
  const lcp::UCell& u = ucell->u;
  // species tables
  std::vector<DevSpecies> sp(nspecies);
  std::vector<double> radial;
  std::vector<int32_t> buckets;
  for (int k = 0; k < nspecies; ++k) {
    const lcp_pao& p = paos[k];
    if (p.max_l < 0 || p.max_l > 3) return fail(LCP_ENOTSUP, "not support PAO l > 3");
    if (p.num_mesh < 8 || !p.rv || !p.rwf) return fail(LCP_EINVAL, "PAO mesh must have >= 8 points");
    for (int i = 1; i < p.num_mesh; ++i)
      if (!(p.rv[i] > p.rv[i - 1])) return fail(LCP_EINVAL, "Spe_PAO_RV must be strictly increasing");
    DevSpecies d{};
    d.max_l = p.max_l;
    d.nmesh = p.num_mesh;
    d.nrad = 0;
    d.no = 0;
    for (int l = 0; l <= p.max_l; ++l) {
      if (p.num_basis[l] < 0) return fail(LCP_EINVAL, "negative Num_Basis");
      d.nb[l] = p.num_basis[l];
      d.nrad += p.num_basis[l];
      d.no += p.num_basis[l] * (2 * l + 1);
    }
    if (d.no > 64) return fail(LCP_ENOTSUP, "more than 64 orbitals per atom");
    d.rv_off = (int64_t)radial.size();
    radial.insert(radial.end(), p.rv, p.rv + p.num_mesh);
    d.rwf_off = (int64_t)radial.size();
    radial.insert(radial.end(), p.rwf, p.rwf + (size_t)d.nrad * p.num_mesh);
    lcp::append_spline_tables(p.rv, p.rwf, p.num_mesh, p.num_basis, p.max_l, d, radial, buckets);
    sp[k] = d;
  }
  std::vector<int32_t> spe0(u.natom);
  for (int a = 0; a < u.natom; ++a) {
    int k = u.atom2spe[a] - 1;
    if (k < 0 || k >= nspecies) return fail(LCP_EINVAL, "atom2spe out of range");
    if (sp[k].no != u.numorbs[a])
      return fail(LCP_EINVAL, "Total_NumOrbs of atom " + std::to_string(a + 1) + " does not match its species basis");
    spe0[a] = k;
  }
  std::unique_ptr<lcp_orbs> o(new lcp_orbs());
  o->ucell = ucell;
  o->device = ctx->device;
  o->grad = with_grad != 0;
  o->max_no = u.max_numorbs();
  if (o->max_no > 32) return fail(LCP_ENOTSUP, "pair contractions support up to 32 orbitals per atom");
  std::vector<int64_t> phi_off(u.natom + 1, 0);
  for (int a = 0; a < u.natom; ++a)
    phi_off[a + 1] = phi_off[a] + (u.sphere_off[a + 1] - u.sphere_off[a]) * (int64_t)u.numorbs[a];
  o->table_elems = phi_off[u.natom];
  cudaStream_t st = ctx->stream;
  API_CUDA(upload(o->atv, u.atv, st), "upload");
  API_CUDA(upload(o->gxyz, u.gxyz, st), "upload");
  API_CUDA(upload(o->spe, spe0, st), "upload");
  API_CUDA(upload(o->sph_off, u.sphere_off, st), "upload");
  API_CUDA(upload(o->glist, u.glist, st), "upload");
  API_CUDA(upload(o->clist, u.clist, st), "upload");
  API_CUDA(upload(o->phi_off, phi_off, st), "upload");
  API_CUDA(upload(o->numorbs, u.numorbs, st), "upload");
  API_CUDA(upload(o->species, sp, st), "upload");
  API_CUDA(upload(o->radial, radial, st), "upload");
  API_CUDA(upload(o->buckets, buckets, st), "upload");
  DevGeom& g = o->geom;
  g.natom = u.natom;
  for (int d = 0; d < 3; ++d) {
    g.ngrid[d] = u.ngrid[d];
    g.origin[d] = u.origin[d];
    for (int c = 0; c < 3; ++c) g.glat[d * 3 + c] = u.glat[d][c];
  }
  g.gridvol = u.gridvol;
  g.atv = o->atv.as<double>();
  g.gxyz = o->gxyz.as<double>();
  g.spe = o->spe.as<int32_t>();
  g.sph_off = o->sph_off.as<int64_t>();
  g.glist = o->glist.as<int32_t>();
  g.clist = o->clist.as<int32_t>();
  g.phi_off = o->phi_off.as<int64_t>();
  g.numorbs = o->numorbs.as<int32_t>();

  // folded pair lists and 512-entry work items
  const int64_t nu = (int64_t)u.uniq_pair.size();
  std::vector<int32_t> pa(nu), pj(nu), pself(nu);
  std::vector<int64_t> bp(nu), bq(nu);
  std::vector<int64_t> ip, is;
  std::vector<int32_t> ic;
  const int64_t chunk = 512;
  // items of pairs with at most 16 orbitals per atom first, then the others
  // (e.g. the 13-orbital pairs of a cell with some 18-orbital atoms get exact
  // 13-orbital tiles instead of 18)
  std::vector<int64_t> ip_l, is_l;
  std::vector<int32_t> ic_l;
  for (int64_t q = 0; q < nu; ++q) {
    int p = u.uniq_pair[q];
    pa[q] = u.pair_atom[p];
    pj[q] = u.pair_jatom[p];
    bp[q] = u.block_off[p];
    bq[q] = u.block_off[u.partner[p]];
    pself[q] = u.partner[p] == p;
    if (u.numorbs[pa[q]] == 0 || u.numorbs[pj[q]] == 0) continue;
    const int no = std::max(u.numorbs[pa[q]], u.numorbs[pj[q]]);
    const bool small = no <= 16;
    if (small) o->max_no_small = std::max(o->max_no_small, no);
    else o->max_no_large = std::max(o->max_no_large, no);
    for (int64_t s0 = u.uniq_off[q]; s0 < u.uniq_off[q + 1]; s0 += chunk) {
      (small ? ip : ip_l).push_back(q);
      (small ? is : is_l).push_back(s0);
      (small ? ic : ic_l).push_back((int32_t)std::min<int64_t>(chunk, u.uniq_off[q + 1] - s0));
    }
  }
  o->nitems_small = (int64_t)ip.size();
  ip.insert(ip.end(), ip_l.begin(), ip_l.end());
  is.insert(is.end(), is_l.begin(), is_l.end());
  ic.insert(ic.end(), ic_l.begin(), ic_l.end());
  API_CUDA(upload(o->p_atom, pa, st), "upload");
  API_CUDA(upload(o->p_jatom, pj, st), "upload");
  API_CUDA(upload(o->p_boffp, bp, st), "upload");
  API_CUDA(upload(o->p_boffq, bq, st), "upload");
  API_CUDA(upload(o->p_self, pself, st), "upload");
  API_CUDA(upload(o->p_lensoff, u.uniq_off, st), "upload");
  API_CUDA(upload(o->p_g1, u.uniq_g1, st), "upload");
  API_CUDA(upload(o->p_g2, u.uniq_g2, st), "upload");
  API_CUDA(upload(o->it_pair, ip, st), "upload");
  API_CUDA(upload(o->it_start, is, st), "upload");
  API_CUDA(upload(o->it_count, ic, st), "upload");
  if (o->grad) {
    // the force term's per-atom entries: item k's kept orientation goes to
    // its pair's atom, the partner orientation to the neighbour atom
    std::vector<int64_t> cnt(u.natom + 1, 0), code;
    for (size_t k = 0; k < ip.size(); ++k) {
      cnt[pa[ip[k]] + 1]++;
      if (!pself[ip[k]]) cnt[pj[ip[k]] + 1]++;
    }
    for (int a = 0; a < u.natom; ++a) cnt[a + 1] += cnt[a];
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    code.resize(cnt[u.natom]);
    for (size_t k = 0; k < ip.size(); ++k) {
      code[fill[pa[ip[k]]]++] = (int64_t)k * 2;
      if (!pself[ip[k]]) code[fill[pj[ip[k]]]++] = (int64_t)k * 2 + 1;
    }
    API_CUDA(upload(o->f_off, cnt, st), "upload");
    API_CUDA(upload(o->f_code, code, st), "upload");
  }
  DevPairs& pr = o->pairs;
  pr.nu = nu;
  pr.atom = o->p_atom.as<int32_t>();
  pr.jatom = o->p_jatom.as<int32_t>();
  pr.boff_p = o->p_boffp.as<int64_t>();
  pr.boff_q = o->p_boffq.as<int64_t>();
  pr.self = o->p_self.as<int32_t>();
  pr.lens_off = o->p_lensoff.as<int64_t>();
  pr.g1 = o->p_g1.as<int32_t>();
  pr.g2 = o->p_g2.as<int32_t>();
  pr.hsize = u.total_hsize;
  pr.nitems = (int64_t)ip.size();
  pr.item_pair = o->it_pair.as<int64_t>();
  pr.item_start = o->it_start.as<int64_t>();
  pr.item_count = o->it_count.as<int32_t>();

  // tabulation
  API_CUDA(o->phi.ensure(o->table_elems * sizeof(double)), "phi alloc");
  if (o->grad)
    for (int k = 0; k < 3; ++k) API_CUDA(o->dphi[k].ensure(o->table_elems * sizeof(double)), "dphi alloc");
  std::vector<int32_t> batom;
  std::vector<int64_t> bstart;
  const int tab_chunk = o->grad ? 64 : lcp::kTabBlock;  // points per block of the gradient / value kernel
  for (int a = 0; a < u.natom; ++a)
    for (int64_t k = u.sphere_off[a]; k < u.sphere_off[a + 1]; k += tab_chunk) {
      batom.push_back(a);
      bstart.push_back(k);
    }
  int max_no_spe = 1;
  for (const DevSpecies& d : sp) max_no_spe = std::max(max_no_spe, (int)d.no);
  DBuf d_batom, d_bstart;
  API_CUDA(upload(d_batom, batom, st), "upload");
  API_CUDA(upload(d_bstart, bstart, st), "upload");
  cudaEvent_t te[2];
  API_CUDA(cudaEventCreate(&te[0]), "event");
  API_CUDA(cudaEventCreate(&te[1]), "event");
  API_CUDA(cudaEventRecord(te[0], st), "event");
  API_CUDA(lcp::launch_tabulate(g, o->species.as<DevSpecies>(), o->radial.as<double>(), o->buckets.as<int32_t>(),
                                (int64_t)batom.size(), d_batom.as<int32_t>(), d_bstart.as<int64_t>(),
                                o->phi.as<double>(), o->grad ? o->dphi[0].as<double>() : nullptr,
                                o->grad ? o->dphi[1].as<double>() : nullptr,
                                o->grad ? o->dphi[2].as<double>() : nullptr, max_no_spe, st),
           "tabulate kernel");
  ctx->launches++;
  API_CUDA(cudaEventRecord(te[1], st), "event");
  API_CUDA(cudaStreamSynchronize(st), "tabulate");
  cudaEventElapsedTime(&o->tab_ms, te[0], te[1]);
  cudaEventDestroy(te[0]);
  cudaEventDestroy(te[1]);
  *out = o.release();
  return LCP_OK;
}

void lcp_orbs_destroy(lcp_orbs* orbs) {
  if (!orbs) return;
  cudaSetDevice(orbs->device);
  delete orbs;
}


lcp_status lcp_orbs_set_brick_shape(lcp_ctx* ctx, lcp_orbs* orbs, const int32_t* shape) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!orbs) return fail(LCP_EINVAL, "NULL orbs");
  int32_t sh[3] = {0, 0, 0};
  if (shape && shape[0] > 0) {
    const int32_t* ng = orbs->ucell->u.ngrid;
    for (int d = 0; d < 3; ++d) {
      if (shape[d] < 1 || shape[d] > 8 || shape[d] > ng[d]) return fail(LCP_EINVAL, "brick sides are 1..min(8, Ngrid)");
      sh[d] = shape[d];
    }
    if (sh[0] * sh[1] * sh[2] > 128) return fail(LCP_EINVAL, "a brick holds at most 128 points");
  }
  if (orbs->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "set brick shape");
  std::memcpy(orbs->brick_shape, sh, sizeof(sh));
  drop_bricks(orbs);
  return LCP_OK;
}

lcp_status lcp_orbs_get_brick_shape(lcp_ctx* ctx, lcp_orbs* orbs, int32_t* shape) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!orbs || !shape) return fail(LCP_EINVAL, "NULL argument");
  if ((s = ensure_bricks(ctx, orbs))) return s;
  for (int d = 0; d < 3; ++d) shape[d] = orbs->bricks.bdim[d];
  return LCP_OK;
}

lcp_status lcp_orbs_release_fp64(lcp_ctx* ctx, lcp_orbs* orbs) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!orbs) return fail(LCP_EINVAL, "NULL orbs");
  if ((s = ensure_bricks(ctx, orbs))) return s;
  API_CUDA(cudaStreamSynchronize(ctx->stream), "release");
  for (DBuf* d : {&orbs->phi, &orbs->dphi[0], &orbs->dphi[1], &orbs->dphi[2], &orbs->phi32}) d->release();
  orbs->phi_released = true;
  return LCP_OK;
}

lcp_status lcp_orbs_autotune_bricks(lcp_ctx* ctx, lcp_orbs* orbs, int32_t ncand, int32_t* shape_out,
                                    double* ms_out) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!orbs || ncand < 1) return fail(LCP_EINVAL, "lcp_orbs_autotune_bricks: NULL orbs or ncand < 1");
  if (orbs->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released");
  const lcp::UCell& u = orbs->ucell->u;
  auto cand = lcp::brick_shape_candidates(u, nullptr);
  // D = V = 1: the passes' work does not depend on the values
  DBuf dm, vp, rho, hk;
  API_CUDA(dm.ensure(u.total_hsize * sizeof(double)), "alloc");
  API_CUDA(hk.ensure(u.total_hsize * sizeof(double)), "alloc");
  API_CUDA(vp.ensure(u.nn() * sizeof(double)), "alloc");
  API_CUDA(rho.ensure(u.nn() * sizeof(double)), "alloc");
  fill_kernel<<<1024, 256, 0, ctx->stream>>>(dm.as<double>(), u.total_hsize, 1.0);
  fill_kernel<<<1024, 256, 0, ctx->stream>>>(vp.as<double>(), u.nn(), 1.0);
  API_CUDA(cudaGetLastError(), "fill");
  const double* cdm[1] = {dm.as<double>()};
  double* prho[1] = {rho.as<double>()};
  const double* cvp[1] = {vp.as<double>()};
  double* phk[1] = {hk.as<double>()};
  cudaEvent_t e0, e1;
  API_CUDA(cudaEventCreate(&e0), "event");
  API_CUDA(cudaEventCreate(&e1), "event");
  double best_ms = 1e30;
  std::array<int32_t, 3> best{0, 0, 0};
  int tried = 0;
  for (size_t i = 0; i < cand.size() && tried < ncand && s == LCP_OK; ++i) {
    std::memcpy(orbs->brick_shape, cand[i].data(), sizeof(int32_t) * 3);
    drop_bricks(orbs);
    lcp_status bs = ensure_bricks(ctx, orbs);
    if (bs == LCP_ENOTSUP) continue;  // too many images per brick for this shape
    if ((s = bs)) break;
    ++tried;
    double ms = 1e30;
    for (int rep = 0; rep < 4 && s == LCP_OK; ++rep) {  // the first run warms up
      cudaEventRecord(e0, ctx->stream);
      if ((s = density_tc_device(ctx, orbs, 1, cdm, prho))) break;
      if ((s = hamiltonian_tc_device(ctx, orbs, 1, cvp, phk))) break;
      cudaEventRecord(e1, ctx->stream);
      cudaError_t e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) {
        s = cuda_fail(e, "autotune");
        break;
      }
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0) ms = std::min(ms, (double)t);
    }
    if (s == LCP_OK && (s = device_status(ctx)) == LCP_OK && ms < best_ms) {
      best_ms = ms;
      best = cand[i];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s) return s;
  if (tried == 0) return fail(LCP_ENOTSUP, "no brick shape keeps the atom images per brick within the limit");
  if (std::memcmp(orbs->bricks.bdim, best.data(), sizeof(int32_t) * 3) != 0 || !orbs->bricks_ready) {
    std::memcpy(orbs->brick_shape, best.data(), sizeof(int32_t) * 3);
    drop_bricks(orbs);
    if ((s = ensure_bricks(ctx, orbs))) return s;
  }
  if (shape_out)
    for (int d = 0; d < 3; ++d) shape_out[d] = best[d];
  if (ms_out) *ms_out = best_ms;
  return LCP_OK;
}

lcp_status lcp_orbs_download(lcp_ctx* ctx, const lcp_orbs* orbs, int32_t component, int32_t atom, double* dst,
                             int64_t count) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!orbs || !dst) return fail(LCP_EINVAL, "NULL argument");
  const lcp::UCell& u = orbs->ucell->u;
  if (atom < 0 || atom >= u.natom) return fail(LCP_EINVAL, "atom index out of range");
  if (component < 0 || component > 3) return fail(LCP_EINVAL, "component must be 0..3");
  if (component > 0 && !orbs->grad) return fail(LCP_ESTATE, "gradient tables were not requested");
  int64_t n = (u.sphere_off[atom + 1] - u.sphere_off[atom]) * (int64_t)u.numorbs[atom];
  if (count != n) return fail(LCP_EINVAL, "count must be GridN*NumOrbs = " + std::to_string(n));
  int64_t off = 0;
  for (int a = 0; a < atom; ++a) off += (u.sphere_off[a + 1] - u.sphere_off[a]) * (int64_t)u.numorbs[a];
  if (orbs->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released");
  const DBuf& b = component == 0 ? orbs->phi : orbs->dphi[component - 1];
  API_CUDA(cudaMemcpyAsync(dst, b.as<double>() + off, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
           "download");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "download");
  return LCP_OK;
}

// ---------------------------------------------------------------- density / H (host buffers)

lcp_status lcp_set_density_grid(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs, int32_t spinpol,
                                const double* const* dm, double* const* density_grid) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if ((s = check_pair(ucell, orbs))) return s;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol.");
  if (!dm || !density_grid) return fail(LCP_EINVAL, "NULL argument");
  const int ns = channels(spinpol);
  const lcp::UCell& u = ucell->u;
  const int64_t nn = u.nn(), hs = u.total_hsize;
  const double* ddm[4];
  double* drho[4];
  for (int c = 0; c < ns; ++c) {
    if (!dm[c] || !density_grid[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[c].ensure(hs * sizeof(double)), "alloc");
    API_CUDA(ctx->w_out[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, dm[c], hs * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    ddm[c] = ctx->w_in[c].as<double>();
    drho[c] = ctx->w_out[c].as<double>();
  }
  if ((s = density_device(ctx, orbs, ns, ddm, drho, nn))) return s;
  for (int c = 0; c < ns; ++c)
    API_CUDA(cudaMemcpyAsync(density_grid[c], drho[c], nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "density");
  return device_status(ctx);
}

lcp_status lcp_calc_matrix_elements(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs, int32_t spinpol,
                                    const double* const* vpot, double* const* hks) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if ((s = check_pair(ucell, orbs))) return s;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol.");
  if (!vpot || !hks) return fail(LCP_EINVAL, "NULL argument");
  const int nc = channels(spinpol);
  const lcp::UCell& u = ucell->u;
  const int64_t nn = u.nn(), hs = u.total_hsize;
  const double* dv[4];
  double* dh[4];
  for (int c = 0; c < nc; ++c) {
    if (!vpot[c] || !hks[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(ctx->w_out[c].ensure(hs * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, vpot[c], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    dv[c] = ctx->w_in[c].as<double>();
    dh[c] = ctx->w_out[c].as<double>();
  }
  if ((s = hamiltonian_device(ctx, orbs, nc, dv, dh, hs))) return s;
  for (int c = 0; c < nc; ++c)
    API_CUDA(cudaMemcpyAsync(hks[c], dh[c], hs * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "hamiltonian");
  return device_status(ctx);
}

// ---------------------------------------------------------------- Poisson / xc / energies (host buffers)

lcp_status lcp_calc_force3(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs, int32_t spinpol,
                           const double* const* vpot, const double* const* dm, double* force) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if ((s = check_pair(ucell, orbs))) return s;
  if (!vpot || !dm || !force) return fail(LCP_EINVAL, "NULL argument");
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "SpinPol must be off, on or nc");
  if (!orbs->grad)
    return fail(LCP_ESTATE, "the force term needs the gradient tables: tabulate with Set_dOrbitals_Grid");
  if (orbs->phi_released) return fail(LCP_ESTATE, "the FP64 orbital tables were released");
  const lcp::UCell& u = ucell->u;
  const int nch = channels(spinpol);
  const double coef[3][4] = {{4, 0, 0, 0}, {2, 2, 0, 0}, {2, 2, 4, -4}};  // src/Force.jl:443-445, 491-493, 554-556
  const double* w = coef[spinpol == LCP_SPIN_OFF ? 0 : (spinpol == LCP_SPIN_ON ? 1 : 2)];
  const int64_t nn = u.nn(), hs = u.total_hsize;
  const double* dv[4];
  const double* dd[4];
  for (int c = 0; c < nch; ++c) {
    if (!vpot[c] || !dm[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(ctx->w_aux[c].ensure(hs * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, vpot[c], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
    API_CUDA(cudaMemcpyAsync(ctx->w_aux[c].p, dm[c], hs * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
    dv[c] = ctx->w_in[c].as<double>();
    dd[c] = ctx->w_aux[c].as<double>();
  }
  const int64_t nitems = orbs->pairs.nitems;
  API_CUDA(ctx->w_part.ensure((size_t)std::max<int64_t>(nitems, 1) * 6 * sizeof(double)), "alloc");
  API_CUDA(ctx->w_out[0].ensure((size_t)std::max(u.natom, 1) * 3 * sizeof(double)), "alloc");
  const double* dphi[3] = {orbs->dphi[0].as<double>(), orbs->dphi[1].as<double>(), orbs->dphi[2].as<double>()};
  int nl = 0;
  API_CUDA(for_item_classes(orbs, &nl,
                            [&](const lcp::DevPairs& pr, int max_no, int64_t first) {
                              // item k's six partial sums at w_part[6 k]
                              return lcp::launch_force3_pairs(orbs->geom, pr, nch, orbs->phi.as<double>(), dphi, dv,
                                                              dd, w, ctx->w_part.as<double>() + 6 * first, max_no,
                                                              ctx->stream);
                            }),
           "force3");
  API_CUDA(lcp::launch_force3_reduce(u.natom, orbs->f_off.as<int64_t>(), orbs->f_code.as<int64_t>(),
                                     ctx->w_part.as<double>(), u.gridvol, ctx->w_out[0].as<double>(), ctx->stream),
           "force3 reduce");
  ctx->launches += nl + 1;
  API_CUDA(cudaMemcpyAsync(force, ctx->w_out[0].p, (size_t)u.natom * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "force3");
  return LCP_OK;
}

static lcp_status check_grid(const int32_t* ng) {
  if (!ng) return fail(LCP_EINVAL, "NULL Ngrid");
  for (int d = 0; d < 3; ++d)
    if (ng[d] <= 0) return fail(LCP_EINVAL, "Ngrid entries must be positive");
  return LCP_OK;
}

static lcp_status poisson_host(lcp_ctx* ctx, const int32_t* ng, const double* recvecs, double* dvhart) {
  const int64_t nn = (int64_t)ng[0] * ng[1] * ng[2];
  const int64_t nspec = (int64_t)ng[0] * ng[1] * (ng[2] / 2 + 1);
  FftPlans* pl = nullptr;
  lcp_status s = get_plans(ctx, ng, &pl);
  if (s) return s;
  API_CUDA(ctx->w_spec.ensure(nspec * 2 * sizeof(double)), "alloc");
  API_CUDA(ctx->w_a.ensure(nn * sizeof(double)), "alloc");
  if ((s = poisson_device(ctx, pl, ng, recvecs, ctx->w_real.as<double>(), ctx->w_spec.p, ctx->w_a.as<double>())))
    return s;
  API_CUDA(cudaMemcpyAsync(dvhart, ctx->w_a.p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "poisson");
  return LCP_OK;
}

lcp_status lcp_solve_poisson_xyz(lcp_ctx* ctx, const int32_t* ngrid, const double* recvecs, const double* density_xyz,
                                 double* dvhart_grid) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if ((s = check_grid(ngrid))) return s;
  if (!recvecs || !density_xyz || !dvhart_grid) return fail(LCP_EINVAL, "NULL argument");
  const int64_t nn = (int64_t)ngrid[0] * ngrid[1] * ngrid[2];
  API_CUDA(ctx->w_real.ensure(nn * sizeof(double)), "alloc");
  API_CUDA(cudaMemcpyAsync(ctx->w_real.p, density_xyz, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
  return poisson_host(ctx, ngrid, recvecs, dvhart_grid);
}

lcp_status lcp_solve_poisson(lcp_ctx* ctx, const int32_t* ngrid, const double* recvecs, int32_t spinpol,
                             const double* const* density_grid, const double* adensity_grid, double* dvhart_grid) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if ((s = check_grid(ngrid))) return s;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol.");
  if (!recvecs || !density_grid || !density_grid[0] || !dvhart_grid) return fail(LCP_EINVAL, "NULL argument");
  if (spinpol != LCP_SPIN_OFF && !density_grid[1]) return fail(LCP_EINVAL, "NULL spin channel");
  const int64_t nn = (int64_t)ngrid[0] * ngrid[1] * ngrid[2];
  const int nr = spinpol == LCP_SPIN_OFF ? 1 : 2;
  for (int c = 0; c < nr; ++c) {
    API_CUDA(ctx->w_in[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, density_grid[c], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
  }
  const double* ad = nullptr;
  if (adensity_grid) {
    API_CUDA(ctx->w_b.ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_b.p, adensity_grid, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    ad = ctx->w_b.as<double>();
  }
  API_CUDA(ctx->w_real.ensure(nn * sizeof(double)), "alloc");
  API_CUDA(lcp::launch_poisson_prep(spinpol, nn, ctx->w_in[0].as<double>(), nr > 1 ? ctx->w_in[1].as<double>() : nullptr,
                                    ad, ctx->w_real.as<double>(), ctx->stream),
           "poisson_prep");
  ctx->launches++;
  return poisson_host(ctx, ngrid, recvecs, dvhart_grid);
}

lcp_status lcp_set_xc_grid(lcp_ctx* ctx, int32_t xc, int32_t spinpol, int64_t nn, const double* pcc,
                           const double* const* density_grid, double* const* vxc_grid) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (xc == LCP_XC_GGA_PBE) return fail(LCP_EINVAL, "GGA_PBE needs the grid: use lcp_set_xc_grid_gga");
  if (xc != LCP_XC_LDA && xc != LCP_XC_LSDA) return fail(LCP_EINVAL, "please check xc_type name");
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol name");
  if ((xc == LCP_XC_LDA) != (spinpol == LCP_SPIN_OFF)) return fail(LCP_EINVAL, "please check xc_type and SpinPol");
  if (nn <= 0 || !density_grid || !vxc_grid) return fail(LCP_EINVAL, "NULL argument");
  const int nr = channels(spinpol);
  const double* dr[4];
  double* dv[4];
  for (int c = 0; c < nr; ++c) {
    if (!density_grid[c] || !vxc_grid[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(ctx->w_out[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, density_grid[c], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
    dr[c] = ctx->w_in[c].as<double>();
    dv[c] = ctx->w_out[c].as<double>();
  }
  const double* dp = nullptr;
  if (pcc) {
    API_CUDA(ctx->w_b.ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_b.p, pcc, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    dp = ctx->w_b.as<double>();
  }
  API_CUDA(lcp::launch_xc_vpot(xc, spinpol, nn, dp, dr, nullptr, nullptr, dv, nullptr, ctx->stream), "xc");
  ctx->launches++;
  for (int c = 0; c < nr; ++c)
    API_CUDA(cudaMemcpyAsync(vxc_grid[c], dv[c], nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "xc");
  return LCP_OK;
}

lcp_status lcp_diagonalize_nc_density(lcp_ctx* ctx, int64_t nn, double* const* density_grid) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (nn <= 0 || !density_grid) return fail(LCP_EINVAL, "NULL argument");
  double* d[4];
  for (int c = 0; c < 4; ++c) {
    if (!density_grid[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, density_grid[c], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
    d[c] = ctx->w_in[c].as<double>();
  }
  API_CUDA(lcp::launch_nc_diagonalize(nn, d, ctx->stream), "nc diagonalize");
  ctx->launches++;
  for (int c = 0; c < 4; ++c)
    API_CUDA(cudaMemcpyAsync(density_grid[c], d[c], nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "nc diagonalize");
  return LCP_OK;
}

lcp_status lcp_calc_diff_coef(const double* glatvecs, double* diff_coef) {
  if (!glatvecs || !diff_coef) return fail(LCP_EINVAL, "NULL argument");
  double gtv[3][3];
  for (int i = 0; i < 3; ++i)
    for (int d = 0; d < 3; ++d) gtv[i][d] = glatvecs[i * 3 + d];
  if (!lcp::calc_diff_coef(gtv, diff_coef)) return fail(LCP_EINVAL, "singular gradient stencil (check gLatvecs)");
  return LCP_OK;
}

// Uploads the GGA inputs into the context's workspaces and fills the cell:
// rho (1 or 2 spins; "nc" angles into w_in[2..3]), pcc, the stencil weights,
// the dE/d(grad rho) scratch and, if wanted, the gradient output.
static lcp_status gga_cell_host(lcp_ctx* ctx, int32_t spinpol, const int32_t* ngrid, const double* dc,
                                const double* pcc, const double* const* density, bool want_dden, lcp::GridCell& c) {
  const int64_t nn = (int64_t)ngrid[0] * ngrid[1] * ngrid[2];
  const int nin = spinpol == LCP_SPIN_OFF ? 1 : (spinpol == LCP_SPIN_ON ? 2 : 4);
  const int ns = spinpol == LCP_SPIN_OFF ? 1 : 2;
  c = lcp::GridCell{};
  for (int d = 0; d < 3; ++d) c.ng[d] = ngrid[d];
  c.nn = nn;
  for (int k = 0; k < nin; ++k) {
    if (!density[k]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[k].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[k].p, density[k], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
  }
  for (int k = 0; k < ns; ++k) {
    c.rho[k] = ctx->w_in[k].as<double>();
    API_CUDA(ctx->w_out[k].ensure(nn * sizeof(double)), "alloc");
    c.vpot[k] = ctx->w_out[k].as<double>();
  }
  if (pcc) {
    API_CUDA(ctx->w_b.ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_b.p, pcc, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    c.pcc = ctx->w_b.as<double>();
  }
  API_CUDA(ctx->w_a.ensure(81 * sizeof(double)), "alloc");
  API_CUDA(cudaMemcpyAsync(ctx->w_a.p, dc, 81 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
  c.dcoef = ctx->w_a.as<double>();
  API_CUDA(ctx->w_aux[0].ensure((size_t)3 * ns * nn * sizeof(double)), "alloc");
  c.dexc = ctx->w_aux[0].as<double>();
  if (want_dden) {
    API_CUDA(ctx->w_aux[1].ensure((size_t)3 * ns * nn * sizeof(double)), "alloc");
    c.dden = ctx->w_aux[1].as<double>();
  }
  return LCP_OK;
}

lcp_status lcp_set_xc_grid_gga(lcp_ctx* ctx, int32_t spinpol, const int32_t* ngrid, const double* diff_coef,
                               const double* pcc, const double* const* density_grid, double* const* vxc_grid,
                               double* const* ddensity_grid, double* const* dexc_dgd) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol name");
  if (!ngrid || !diff_coef || !density_grid || !vxc_grid) return fail(LCP_EINVAL, "NULL argument");
  if (ngrid[0] <= 0 || ngrid[1] <= 0 || ngrid[2] <= 0) return fail(LCP_EINVAL, "Ngrid must be positive");
  const int64_t nn = (int64_t)ngrid[0] * ngrid[1] * ngrid[2];
  const int ns = spinpol == LCP_SPIN_OFF ? 1 : 2;
  const int nv = channels(spinpol);
  for (int k = 0; k < nv; ++k)
    if (!vxc_grid[k]) return fail(LCP_EINVAL, "NULL channel");
  lcp::GridCell c;
  if ((s = gga_cell_host(ctx, spinpol, ngrid, diff_coef, pcc, density_grid, ddensity_grid != nullptr, c))) return s;
  API_CUDA(lcp::launch_gga_g(spinpol, c, lcp::GridBatch{}, true, ctx->xc_dfl != 0, ctx->stream), "gga");
  ctx->launches += 2;
  if (spinpol == LCP_SPIN_NC) {
    for (int k = 2; k < 4; ++k) API_CUDA(ctx->w_out[k].ensure(nn * sizeof(double)), "alloc");
    double* o[4] = {ctx->w_out[0].as<double>(), ctx->w_out[1].as<double>(), ctx->w_out[2].as<double>(),
                    ctx->w_out[3].as<double>()};
    API_CUDA(lcp::launch_nc_rotate(nn, o[0], o[1], ctx->w_in[2].as<double>(), ctx->w_in[3].as<double>(), -1.0, o,
                                   ctx->stream),
             "gga nc");
    ctx->launches++;
  }
  for (int k = 0; k < nv; ++k)
    API_CUDA(cudaMemcpyAsync(vxc_grid[k], ctx->w_out[k].p, nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
             "D2H");
  for (int k = 0; k < 3 * ns; ++k) {
    if (ddensity_grid && ddensity_grid[k])
      API_CUDA(cudaMemcpyAsync(ddensity_grid[k], c.dden + k * nn, nn * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream),
               "D2H");
    if (dexc_dgd && dexc_dgd[k])
      API_CUDA(cudaMemcpyAsync(dexc_dgd[k], c.dexc + k * nn, nn * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream),
               "D2H");
  }
  API_CUDA(cudaStreamSynchronize(ctx->stream), "gga");
  return LCP_OK;
}

lcp_status lcp_set_vpot_grid(lcp_ctx* ctx, int32_t spinpol, int64_t nn, const double* dvhart, const double* const* vxc,
                             const double* vna, double* const* vpot) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol");
  if (nn <= 0 || !dvhart || !vxc || !vpot) return fail(LCP_EINVAL, "NULL argument");
  const int nv = channels(spinpol);
  const double* dx[4];
  double* dp[4];
  API_CUDA(ctx->w_a.ensure(nn * sizeof(double)), "alloc");
  API_CUDA(cudaMemcpyAsync(ctx->w_a.p, dvhart, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
  for (int c = 0; c < nv; ++c) {
    if (!vxc[c] || !vpot[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(ctx->w_out[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, vxc[c], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    dx[c] = ctx->w_in[c].as<double>();
    dp[c] = ctx->w_out[c].as<double>();
  }
  const double* dn = nullptr;
  if (vna) {
    API_CUDA(ctx->w_b.ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_b.p, vna, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    dn = ctx->w_b.as<double>();
  }
  API_CUDA(lcp::launch_vpot(spinpol, nn, ctx->w_a.as<double>(), dx, dn, dp, ctx->stream), "vpot");
  ctx->launches++;
  for (int c = 0; c < nv; ++c)
    API_CUDA(cudaMemcpyAsync(vpot[c], dp[c], nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "vpot");
  return LCP_OK;
}

static lcp_status energy_host(lcp_ctx* ctx, int32_t xc, int32_t spinpol, int64_t nn, const double* aden,
                              const double* pcc, const double* const* density, const double* dvhart, double out[3]) {
  const int nr = spinpol == LCP_SPIN_OFF ? 1 : 2;
  const double* dr[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int c = 0; c < nr; ++c) {
    if (!density[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(ctx->w_in[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_in[c].p, density[c], nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    dr[c] = ctx->w_in[c].as<double>();
  }
  const double* d_ad = nullptr;
  const double* d_pc = nullptr;
  const double* d_vh = nullptr;
  if (aden) {
    API_CUDA(ctx->w_aux[0].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_aux[0].p, aden, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    d_ad = ctx->w_aux[0].as<double>();
  }
  if (pcc) {
    API_CUDA(ctx->w_aux[1].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_aux[1].p, pcc, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    d_pc = ctx->w_aux[1].as<double>();
  }
  if (dvhart) {
    API_CUDA(ctx->w_aux[2].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_aux[2].p, dvhart, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    d_vh = ctx->w_aux[2].as<double>();
  }
  API_CUDA(ctx->w_part.ensure((size_t)std::max<int64_t>(lcp::red_tiles(nn), 1) * 3 * sizeof(double)), "alloc");
  API_CUDA(ctx->w_scal.ensure(8 * sizeof(double)), "alloc");
  API_CUDA(lcp::launch_energy_sums(xc, spinpol, nn, d_ad, d_pc, dr, d_vh, ctx->w_part.as<double>(),
                                   ctx->w_scal.as<double>(), ctx->stream),
           "energy");
  ctx->launches += 2;
  API_CUDA(cudaMemcpyAsync(out, ctx->w_scal.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "energy");
  return LCP_OK;
}

lcp_status lcp_calc_eh1(lcp_ctx* ctx, int32_t spinpol, int64_t nn, double gridvol, const double* adensity,
                        const double* const* density, const double* dvhart, double* eh1) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol");
  if (nn <= 0 || !density || !dvhart || !eh1) return fail(LCP_EINVAL, "NULL argument");
  double out[3];
  if ((s = energy_host(ctx, spinpol == LCP_SPIN_OFF ? LCP_XC_LDA : LCP_XC_LSDA, spinpol, nn, adensity, nullptr, density,
                       dvhart, out)))
    return s;
  *eh1 = out[0] * gridvol * 0.5;
  return LCP_OK;
}

lcp_status lcp_calc_exc1(lcp_ctx* ctx, int32_t xc, int32_t spinpol, int64_t nn, double gridvol, const double* adensity,
                         const double* pcc, const double* const* density, double* exc) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (xc == LCP_XC_GGA_PBE) return fail(LCP_EINVAL, "GGA_PBE needs the grid: use lcp_calc_exc1_grid");
  if (xc != LCP_XC_LDA && xc != LCP_XC_LSDA) return fail(LCP_EINVAL, "please check xc_type");
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol");
  if (nn <= 0 || !density || !exc) return fail(LCP_EINVAL, "NULL argument");
  double out[3];
  if ((s = energy_host(ctx, xc, spinpol, nn, adensity, pcc, density, nullptr, out))) return s;
  exc[0] = out[1] * gridvol;
  exc[1] = out[2] * gridvol;
  return LCP_OK;
}

lcp_status lcp_calc_exc1_grid(lcp_ctx* ctx, int32_t xc, int32_t spinpol, const int32_t* ngrid, const double* latvecs,
                              double gridvol, const double* adensity, const double* pcc, const double* const* density,
                              double* exc) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!ngrid || !density || !exc) return fail(LCP_EINVAL, "NULL argument");
  if (ngrid[0] <= 0 || ngrid[1] <= 0 || ngrid[2] <= 0) return fail(LCP_EINVAL, "Ngrid must be positive");
  const int64_t nn = (int64_t)ngrid[0] * ngrid[1] * ngrid[2];
  if (xc != LCP_XC_GGA_PBE) return lcp_calc_exc1(ctx, xc, spinpol, nn, gridvol, adensity, pcc, density, exc);
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol");
  if (!latvecs) return fail(LCP_EINVAL, "NULL argument");
  double gtv[3][3], dc[81];
  grid_vectors(latvecs, ngrid, gtv);
  if (!lcp::calc_diff_coef(gtv, dc)) return fail(LCP_EINVAL, "singular gradient stencil (check Latvecs)");
  // Calc_EXC1 reads the two collinear spins only, also for "nc"
  const int32_t sp = spinpol == LCP_SPIN_OFF ? LCP_SPIN_OFF : LCP_SPIN_ON;
  lcp::GridCell c;
  if ((s = gga_cell_host(ctx, sp, ngrid, dc, pcc, density, false, c))) return s;
  if (adensity) {
    API_CUDA(ctx->w_aux[2].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(ctx->w_aux[2].p, adensity, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
    c.aden = ctx->w_aux[2].as<double>();
  }
  API_CUDA(ctx->w_part.ensure((size_t)std::max<int64_t>(lcp::red_tiles(nn), 1) * 3 * sizeof(double)), "alloc");
  API_CUDA(ctx->w_scal.ensure(16 * sizeof(double)), "alloc");
  c.part = ctx->w_part.as<double>();
  c.sums = ctx->w_scal.as<double>();
  API_CUDA(lcp::launch_gga_g(sp, c, lcp::GridBatch{}, false, ctx->xc_dfl != 0, ctx->stream), "gga energy");
  API_CUDA(lcp::launch_grid_sums_g(c, lcp::GridBatch{}, ctx->stream), "gga energy sums");
  ctx->launches += 2;
  double out[3];
  API_CUDA(cudaMemcpyAsync(out, ctx->w_scal.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "gga energy");
  exc[0] = out[1] * gridvol;
  exc[1] = out[2] * gridvol;
  return LCP_OK;
}

// ---------------------------------------------------------------- device-resident job

lcp_status lcp_job_create(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs, int32_t spinpol, int32_t xc,
                          const double* adensity, const double* pcc, const double* vna, lcp_job** out) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if ((s = check_pair(ucell, orbs))) return s;
  if (!out) return fail(LCP_EINVAL, "NULL argument");
  *out = nullptr;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol");
  if (xc != LCP_XC_LDA && xc != LCP_XC_LSDA && xc != LCP_XC_GGA_PBE) return fail(LCP_EINVAL, "please check xc_type");
  if (xc != LCP_XC_GGA_PBE && (xc == LCP_XC_LDA) != (spinpol == LCP_SPIN_OFF))
    return fail(LCP_EINVAL, "please check xc_type and SpinPol");
  const lcp::UCell& u = ucell->u;
  std::unique_ptr<lcp_job> j(new lcp_job());
  j->ucell = ucell;
  j->orbs = orbs;
  j->spinpol = spinpol;
  j->xc = xc;
  j->nspin = channels(spinpol);
  j->nn = u.nn();
  j->hsize = u.total_hsize;
  // Recvecs = 2*pi*inv(Latvecs') (src/Mixing/DFT_Mixing.jl:91): rows b_i with a_i.b_j = 2*pi*delta_ij
  {
    const double(&L)[3][3] = u.lat;
    double det = L[0][0] * (L[1][1] * L[2][2] - L[1][2] * L[2][1]) - L[0][1] * (L[1][0] * L[2][2] - L[1][2] * L[2][0]) +
                 L[0][2] * (L[1][0] * L[2][1] - L[1][1] * L[2][0]);
    double c = 2 * 3.14159265358979323846 / det;
    for (int i = 0; i < 3; ++i) {
      int a = (i + 1) % 3, b = (i + 2) % 3;
      j->recvecs[i * 3 + 0] = c * (L[a][1] * L[b][2] - L[a][2] * L[b][1]);
      j->recvecs[i * 3 + 1] = c * (L[a][2] * L[b][0] - L[a][0] * L[b][2]);
      j->recvecs[i * 3 + 2] = c * (L[a][0] * L[b][1] - L[a][1] * L[b][0]);
    }
  }
  const int64_t nn = j->nn, hs = j->hsize;
  const int64_t nspec = (int64_t)u.ngrid[0] * u.ngrid[1] * (u.ngrid[2] / 2 + 1);
  for (int c = 0; c < j->nspin; ++c) {
    API_CUDA(j->dm[c].ensure(hs * sizeof(double)), "alloc");
    API_CUDA(j->hks[c].ensure(hs * sizeof(double)), "alloc");
    API_CUDA(j->rho[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(j->vpot[c].ensure(nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemsetAsync(j->dm[c].p, 0, hs * sizeof(double), ctx->stream), "memset");
  }
  API_CUDA(j->dvh.ensure(nn * sizeof(double)), "alloc");
  API_CUDA(j->real.ensure(nn * sizeof(double)), "alloc");
  API_CUDA(j->spec.ensure(nspec * 2 * sizeof(double)), "alloc");
  API_CUDA(j->part.ensure((size_t)std::max<int64_t>({3 * lcp::red_tiles(nn), lcp::red_tiles(hs), 1}) * sizeof(double)),
           "alloc");
  API_CUDA(j->scal.ensure(16 * sizeof(double)), "alloc");
  API_CUDA(j->pfac.ensure(nspec * sizeof(double)), "alloc");
  API_CUDA(lcp::launch_poisson_table(u.ngrid, j->recvecs, j->pfac.as<double>(), ctx->stream), "poisson table");
  if (xc == LCP_XC_GGA_PBE) {
    double gtv[3][3], dc[81];
    grid_vectors(&u.lat[0][0], u.ngrid, gtv);
    if (!lcp::calc_diff_coef(gtv, dc)) return fail(LCP_EINVAL, "singular gradient stencil (check Latvecs)");
    API_CUDA(j->dcoef.ensure(81 * sizeof(double)), "alloc");
    API_CUDA(j->dexc.ensure((size_t)3 * j->nspin * nn * sizeof(double)), "alloc");
    API_CUDA(cudaMemcpyAsync(j->dcoef.p, dc, sizeof dc, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    API_CUDA(cudaStreamSynchronize(ctx->stream), "H2D");  // dc is a stack buffer
  }
  auto put = [&](DBuf& b, const double* src, bool& flag) -> cudaError_t {
    flag = src != nullptr;
    if (!src) return cudaSuccess;
    cudaError_t e = b.ensure(nn * sizeof(double));
    if (e) return e;
    return cudaMemcpyAsync(b.p, src, nn * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  };
  API_CUDA(put(j->aden, adensity, j->has_aden), "H2D");
  API_CUDA(put(j->pcc, pcc, j->has_pcc), "H2D");
  API_CUDA(put(j->vna, vna, j->has_vna), "H2D");
  if ((s = get_plans(ctx, u.ngrid, &j->plans))) return s;
  API_CUDA(cudaStreamSynchronize(ctx->stream), "job create");
  *out = j.release();
  return LCP_OK;
}

void lcp_job_destroy(lcp_job* job) { delete job; }

lcp_status lcp_job_set_dm(lcp_ctx* ctx, lcp_job* job, const double* const* dm) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!job || !dm) return fail(LCP_EINVAL, "NULL argument");
  for (int c = 0; c < job->nspin; ++c) {
    if (!dm[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(cudaMemcpyAsync(job->dm[c].p, dm[c], job->hsize * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
             "H2D");
  }
  return LCP_OK;
}

static lcp_status job_step_impl(lcp_ctx* ctx, lcp_job* job, cudaEvent_t* ev) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!job) return fail(LCP_EINVAL, "NULL job");
  auto mark = [&](int k) {
    if (ev) cudaEventRecord(ev[k], ctx->stream);
  };
  const lcp::UCell& u = job->ucell->u;
  const int ns = job->nspin;
  cudaStream_t st = ctx->stream;
  const double* dm[4];
  double* rho[4];
  const double* cvp[4];
  double* hk[4];
  for (int c = 0; c < ns; ++c) {
    dm[c] = job->dm[c].as<double>();
    rho[c] = job->rho[c].as<double>();
    cvp[c] = job->vpot[c].as<double>();
    hk[c] = job->hks[c].as<double>();
  }
  const lcp::GridCell gc = job_grid_cell(job);
  const lcp::GridBatch one{};
  // 1. density
  mark(0);
  if ((s = density_device(ctx, job->orbs, ns, dm, rho, job->nn))) return s;
  if (job->spinpol == LCP_SPIN_NC) {
    // diagonalize_nc_density! (src/KSsolve_SCF.jl:252-255): rho[0..3] become Nup, Ndown, theta, phi
    API_CUDA(lcp::launch_nc_diagonalize(job->nn, rho, st), "nc diagonalize");
    ctx->launches++;
  }
  mark(1);
  // The xc pass needs only rho: in an untimed step it runs on the context's
  // second stream beside the FFT Poisson solve (without dVHart: vpot holds
  // vxc), and vpot_eh_g adds dVHart + V_na and the E_H1 partials after both.
  // "nc": the collinear pass on (Nup, Ndown), the rotation afterwards.
  const int32_t sp_xc = job->spinpol == LCP_SPIN_NC ? LCP_SPIN_ON : job->spinpol;
  auto xc_pass = [&](const lcp::GridCell& c, cudaStream_t xs) -> lcp_status {
    if (job->xc == LCP_XC_GGA_PBE) {
      API_CUDA(lcp::launch_gga_g(sp_xc, c, one, true, ctx->precision != LCP_PREC_FP64, xs), "gga");
      ctx->launches += 2;
    } else {
      API_CUDA(lcp::launch_xc_vpot_energy_g(job->xc, sp_xc, c, one, ctx->precision != LCP_PREC_FP64, xs),
               "xc_vpot_energy");
      ctx->launches++;
    }
    return LCP_OK;
  };
  const bool overlap = ev == nullptr;
  if (overlap) {
    if (!ctx->aux) API_CUDA(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!ctx->ev_fork) API_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming), "cudaEventCreate");
    if (!ctx->ev_join) API_CUDA(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming), "cudaEventCreate");
    API_CUDA(cudaEventRecord(ctx->ev_fork, st), "fork");
    API_CUDA(cudaStreamWaitEvent(ctx->aux, ctx->ev_fork, 0), "fork");
    lcp::GridCell gx = gc;
    gx.dvh = nullptr;
    if ((s = xc_pass(gx, ctx->aux))) return s;
    API_CUDA(cudaEventRecord(ctx->ev_join, ctx->aux), "join");
  }
  // 2. Poisson: the hand-written FFT solve, the source formed in its first pass
  FftPlans* plans = nullptr;  // the executing context's plans (any context may run the job)
  if ((s = get_plans(ctx, u.ngrid, &plans))) return s;
  API_CUDA(lcp::launch_poisson_fft(plans->geom, ctx->precision == LCP_PREC_FP64, job->spinpol, gc, nullptr, 1, st),
           "poisson fft");
  ctx->launches += 5;
  mark(2);
  // 3. xc + potential, with the FP64 energy tile partials
  if (overlap) {
    API_CUDA(cudaStreamWaitEvent(st, ctx->ev_join, 0), "join");
    API_CUDA(lcp::launch_vpot_eh_g(sp_xc, gc, one, st), "vpot_eh");
    ctx->launches++;
  } else if ((s = xc_pass(gc, st))) {
    return s;
  }
  if (job->spinpol == LCP_SPIN_NC) {
    // dVHart + V_na is common to both diagonal channels and drops out of tmp1
    double* vp[4] = {job->vpot[0].as<double>(), job->vpot[1].as<double>(), job->vpot[2].as<double>(),
                     job->vpot[3].as<double>()};
    API_CUDA(lcp::launch_nc_rotate(job->nn, vp[0], vp[1], rho[2], rho[3], job->xc == LCP_XC_GGA_PBE ? -1.0 : 1.0, vp,
                                   st),
             "nc rotate");
    ctx->launches++;
  }
  mark(3);
  // 4. FP64 energy terms: the sums of the tile partials
  API_CUDA(lcp::launch_grid_sums_g(gc, one, st), "energy");
  ctx->launches++;
  mark(4);
  // 5. grid matrix elements
  if ((s = hamiltonian_device(ctx, job->orbs, ns, cvp, hk, job->hsize))) return s;
  mark(5);
  // 6. sum_s <D_s, H_s> and the job energies
  API_CUDA(lcp::launch_dot_energy_g(job->spinpol, ns, gc, one, one, st), "dot");
  ctx->launches += 2;
  mark(6);
  return LCP_OK;
}

// What a captured step depends on besides the job's own buffers: the
// context's stream and options, and every device buffer of the library (a
// (re)allocation or a free anywhere moves one of the two counters).
static void step_signature(const lcp_ctx* ctx, int64_t* sig) {
  sig[0] = (int64_t)reinterpret_cast<intptr_t>(ctx->stream);
  sig[1] = ctx->precision;
  sig[2] = ctx->xc_dfl;
  sig[3] = ctx->fault_poll;
  sig[4] = ctx->fault_stall;
  sig[5] = ctx->tc_ev != nullptr;
  sig[6] = g_device_allocs.load(std::memory_order_relaxed);
  sig[7] = g_device_frees.load(std::memory_order_relaxed);
}

// One step.  The first step of a job on a context runs its launches
// directly (and makes every workspace it needs); the next one with the same
// signature captures them into a CUDA graph, which later steps replay with
// one launch: the step's ~20 kernels then reach the GPU at once instead of
// one by one behind the host, which matters after a synchronising read
// (the end-to-end loop: D in, step, H out).  A step that cannot be captured
// (a stream without capture support, an unexpected call) runs without a
// graph from then on.
lcp_status lcp_job_step(lcp_ctx* ctx, lcp_job* job) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!job) return fail(LCP_EINVAL, "NULL job");
  if (!ctx->step_graphs) return job_step_impl(ctx, job, nullptr);
  // a caller capturing the stream gets the launches in its own graph
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  API_CUDA(cudaStreamIsCapturing(ctx->stream, &cap), "capture status");
  if (cap != cudaStreamCaptureStatusNone) return job_step_impl(ctx, job, nullptr);
  lcp_job::StepGraph& G = job->graphs[ctx];
  int64_t sig[8];
  step_signature(ctx, sig);
  auto same = [](const int64_t* a, const int64_t* b) { return std::equal(a, a + 8, b); };
  if (G.exec && same(G.sig, sig)) {
    API_CUDA(cudaGraphLaunch(G.exec, ctx->stream), "graph launch");
    ctx->launches += G.launches;
    return LCP_OK;
  }
  if (G.exec) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  if (!G.off && G.have_prev && same(G.prev, sig)) {
    const int64_t l0 = ctx->launches;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      s = job_step_impl(ctx, job, nullptr);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
      int64_t after[8];
      step_signature(ctx, after);
      cudaGraphExec_t x = nullptr;
      if (s == LCP_OK && e == cudaSuccess && g && same(after, sig) && cudaGraphInstantiate(&x, g, 0) == cudaSuccess) {
        cudaGraphDestroy(g);
        std::copy(sig, sig + 8, G.sig);
        G.exec = x;
        G.launches = ctx->launches - l0;
        API_CUDA(cudaGraphLaunch(x, ctx->stream), "graph launch");
        return LCP_OK;
      }
      if (g) cudaGraphDestroy(g);
    }
    (void)cudaGetLastError();  // the failed capture's error, if any
    G.off = true;
    ctx->launches = l0;
  }
  s = job_step_impl(ctx, job, nullptr);
  step_signature(ctx, G.prev);
  G.have_prev = true;
  return s;
}

lcp_status lcp_ctx_set_step_graphs(lcp_ctx* ctx, int32_t on) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (on < 0 || on > 1) return fail(LCP_EINVAL, "on is 0 or 1");
  ctx->step_graphs = on;
  return LCP_OK;
}

lcp_status lcp_job_step_timed(lcp_ctx* ctx, lcp_job* job, double* stage_ms) {
  if (!stage_ms) return fail(LCP_EINVAL, "NULL argument");
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  cudaEvent_t ev[7];
  for (int k = 0; k < 7; ++k) API_CUDA(cudaEventCreate(&ev[k]), "cudaEventCreate");
  s = job_step_impl(ctx, job, ev);
  if (s == LCP_OK) {
    cudaError_t e = cudaEventSynchronize(ev[6]);
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) {
      float ms = 0.f;
      e = cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
      stage_ms[k] = ms;
    }
    if (e != cudaSuccess) s = cuda_fail(e, "stage timing");
  }
  for (int k = 0; k < 7; ++k) cudaEventDestroy(ev[k]);
  return s;
}

lcp_status lcp_job_tc_kernel_ms(lcp_ctx* ctx, lcp_job* job, double* out2) {
  if (!out2) return fail(LCP_EINVAL, "NULL argument");
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (ctx->precision != LCP_PREC_BF16X3) return fail(LCP_ENOTSUP, "the tensor-core kernels run in split-BF16 only");
  cudaEvent_t ev[16];
  int made = 0;
  for (; made < 16; ++made)
    if (cudaEventCreate(&ev[made]) != cudaSuccess) break;
  if (made < 16) {
    for (int k = 0; k < made; ++k) cudaEventDestroy(ev[k]);
    return fail(LCP_EDEVICE, "cudaEventCreate");
  }
  ctx->tc_ev = ev;
  s = job_step_impl(ctx, job, nullptr);
  ctx->tc_ev = nullptr;
  double sum[2] = {0.0, 0.0};
  if (s == LCP_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    const int nd = job->nspin, nh = job->spinpol == LCP_SPIN_NC ? 4 : job->nspin;
    for (int k = 0; k < 2 && e == cudaSuccess; ++k)
      for (int c = 0; c < (k ? nh : nd) && e == cudaSuccess; ++c) {
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, ev[8 * k + 2 * c], ev[8 * k + 2 * c + 1]);
        sum[k] += ms;
      }
    if (e != cudaSuccess) s = cuda_fail(e, "tensor-core kernel timing");
  }
  for (int k = 0; k < 16; ++k) cudaEventDestroy(ev[k]);
  out2[0] = sum[0];
  out2[1] = sum[1];
  return s;
}

lcp_status lcp_job_energies(lcp_ctx* ctx, lcp_job* job, double* out5) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!job || !out5) return fail(LCP_EINVAL, "NULL argument");
  API_CUDA(cudaMemcpyAsync(out5, job->scal.as<double>() + 8, 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
           "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "energies");
  return device_status(ctx);
}

lcp_status lcp_job_energies_async(lcp_ctx* ctx, lcp_job* job, double* out5) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!job || !out5) return fail(LCP_EINVAL, "NULL argument");
  API_CUDA(cudaMemcpyAsync(out5, job->scal.as<double>() + 8, 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
           "D2H");
  return LCP_OK;
}

lcp_status lcp_job_footprint(const lcp_job* job, int64_t* bytes) {
  if (!job || !bytes) return fail(LCP_EINVAL, "NULL argument");
  int64_t b = 0;
  auto add = [&](const DBuf& d) { b += (int64_t)d.bytes; };
  for (int c = 0; c < 4; ++c) {
    add(job->dm[c]);
    add(job->rho[c]);
    add(job->hks[c]);
    add(job->vpot[c]);
  }
  for (const DBuf* d : {&job->aden, &job->pcc, &job->vna, &job->dvh, &job->real, &job->spec, &job->part, &job->scal,
                        &job->pfac, &job->dcoef, &job->dexc})
    add(*d);
  const lcp_orbs* o = job->orbs;
  for (const DBuf* d : {&o->atv, &o->gxyz, &o->spe, &o->sph_off, &o->glist, &o->clist, &o->phi_off, &o->numorbs,
                        &o->species, &o->radial, &o->phi, &o->dphi[0], &o->dphi[1], &o->dphi[2], &o->phi32,
                        &o->p_atom, &o->p_jatom, &o->p_boffp, &o->p_boffq, &o->p_self, &o->p_lensoff, &o->p_g1,
                        &o->p_g2, &o->it_pair, &o->it_start, &o->it_count, &o->f_off, &o->f_code, &o->b_code, &o->b_imgoff, &o->b_imgblk,
                        &o->b_taboff, &o->b_tabpair, &o->b_tab, &o->b_tabslot, &o->b_slotbase, &o->b_redoff,
                        &o->b_redslot, &o->b_subpair, &o->b_subchunks, &o->b_sbfold, &o->b_sbchunks, &o->o_atom,
                        &o->o_jatom, &o->o_boff, &o->o_partner, &o->b_scale, &o->b_tmp})
    add(*d);
  *bytes = b;
  return LCP_OK;
}

}  // extern "C"

// Device bytes the job will hold once its tables for `precision` exist: its
// footprint now plus, when not built yet, the split-BF16 brick tables (from
// the host brick geometry) or the FP32 orbital copy.
int64_t job_footprint_estimate(lcp_job* job, int32_t precision) {
  int64_t fp = 0;
  if (lcp_job_footprint(job, &fp) != LCP_OK) return -1;
  const lcp_orbs* o = job->orbs;
  if (precision == LCP_PREC_BF16X3 && !o->bricks_ready) {
    lcp::Bricks b;
    if (!lcp::build_bricks(o->ucell->u, b, o->brick_shape[0] > 0 ? o->brick_shape : nullptr).empty()) return -1;
    fp += b.nblocks * 6144 * 2 + (int64_t)b.point_code.size() * 4 + (int64_t)b.tab_pair.size() * 8 +
          (int64_t)(b.img_off.size() + b.slot_base.size() + b.red_off.size() + b.red_slot.size()) * 8 +
          (int64_t)(b.img_block.size() + b.sub_pair.size() + b.sub_chunks.size() + b.sb_fold.size() +
                    b.sb_chunks.size()) * 4;
  } else if (precision == LCP_PREC_FP32 && !o->phi32.p) {
    fp += o->table_elems * 4;
  }
  return fp;
}

extern "C" {

lcp_status lcp_job_prepare(lcp_ctx* ctx, lcp_job* job) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!job) return fail(LCP_EINVAL, "NULL job");
  lcp_orbs* o = const_cast<lcp_orbs*>(job->orbs);
  if (ctx->precision == LCP_PREC_BF16X3) return ensure_bricks(ctx, o);
  if (ctx->precision == LCP_PREC_FP32) {
    if ((s = ensure_phi32(ctx, o))) return s;
    API_CUDA(cudaStreamSynchronize(ctx->stream), "prepare");
  }
  return LCP_OK;
}

lcp_status lcp_ctx_check_status(lcp_ctx* ctx) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  API_CUDA(cudaStreamSynchronize(ctx->stream), "status");
  return device_status(ctx);
}

static lcp_status job_get(lcp_ctx* ctx, lcp_job* job, DBuf* src, int64_t n, double* const* dst) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!job || !dst) return fail(LCP_EINVAL, "NULL argument");
  for (int c = 0; c < job->nspin; ++c) {
    if (!dst[c]) return fail(LCP_EINVAL, "NULL channel");
    API_CUDA(cudaMemcpyAsync(dst[c], src[c].p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  }
  API_CUDA(cudaStreamSynchronize(ctx->stream), "job get");
  return LCP_OK;
}

lcp_status lcp_tc_selftest(lcp_ctx* ctx, int32_t a_mn_major, int32_t b_mn_major, int32_t order, int32_t n,
                           int32_t k, const float* a, const float* b, float* d) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!a || !b || !d) return fail(LCP_EINVAL, "NULL argument");
  if (n < 16 || n > 256 || n % 16 || k < 16 || k > 64 || k % 16) return fail(LCP_EINVAL, "N in 16..256, K in 16..64, multiples of 16");
  DBuf da, db, dd, dst;
  API_CUDA(da.ensure(128 * k * sizeof(float)), "alloc");
  API_CUDA(db.ensure((size_t)n * k * sizeof(float)), "alloc");
  API_CUDA(dd.ensure((size_t)128 * n * sizeof(float)), "alloc");
  API_CUDA(dst.ensure(sizeof(int)), "alloc");
  API_CUDA(cudaMemsetAsync(dst.p, 0, sizeof(int), ctx->stream), "memset");
  API_CUDA(cudaMemcpyAsync(da.p, a, 128 * k * sizeof(float), cudaMemcpyHostToDevice, ctx->stream), "H2D");
  API_CUDA(cudaMemcpyAsync(db.p, b, (size_t)n * k * sizeof(float), cudaMemcpyHostToDevice, ctx->stream), "H2D");
  API_CUDA(lcp::launch_tc_selftest(da.as<float>(), db.as<float>(), dd.as<float>(), n, k, a_mn_major, b_mn_major,
                                   order, dst.as<int>(), ctx->stream),
           "tc selftest");
  ctx->launches++;
  int st = 0;
  API_CUDA(cudaMemcpyAsync(&st, dst.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaMemcpyAsync(d, dd.p, (size_t)128 * n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "tc selftest");
  if (st) return fail(st, "tensor-core self-test: MMA completion wait timed out");
  return LCP_OK;
}

lcp_status lcp_xc_selftest(lcp_ctx* ctx, int32_t xc, int32_t double_float, int64_t n, const double* up,
                           const double* dn, const double* pcc, double* out) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!up || !out || (xc != LCP_XC_LDA && !dn)) return fail(LCP_EINVAL, "NULL argument");
  if (xc != LCP_XC_LDA && xc != LCP_XC_LSDA) return fail(LCP_EINVAL, "xc: LDA or LSDA");
  if (n < 0) return fail(LCP_EINVAL, "n < 0");
  if (n == 0) return LCP_OK;
  DBuf dup, ddn, dpc, dout;
  const size_t b = (size_t)n * sizeof(double);
  API_CUDA(dup.ensure(b), "alloc");
  API_CUDA(dout.ensure(3 * b), "alloc");
  API_CUDA(cudaMemcpyAsync(dup.p, up, b, cudaMemcpyHostToDevice, ctx->stream), "H2D");
  if (xc != LCP_XC_LDA) {
    API_CUDA(ddn.ensure(b), "alloc");
    API_CUDA(cudaMemcpyAsync(ddn.p, dn, b, cudaMemcpyHostToDevice, ctx->stream), "H2D");
  }
  if (pcc) {
    API_CUDA(dpc.ensure(b), "alloc");
    API_CUDA(cudaMemcpyAsync(dpc.p, pcc, b, cudaMemcpyHostToDevice, ctx->stream), "H2D");
  }
  API_CUDA(lcp::launch_xc_selftest(xc, double_float != 0, n, dup.as<double>(), ddn.as<double>(),
                                   pcc ? dpc.as<double>() : nullptr, dout.as<double>(), ctx->stream),
           "xc selftest");
  ctx->launches++;
  API_CUDA(cudaMemcpyAsync(out, dout.p, 3 * b, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "xc selftest");
  return LCP_OK;
}

lcp_status lcp_probe_fp64_tflops(lcp_ctx* ctx, double* tflops) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!tflops) return fail(LCP_EINVAL, "NULL argument");
  int sms = 0;
  API_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "attr");
  DBuf out;
  API_CUDA(out.ensure(64), "alloc");
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t a, b;
  API_CUDA(cudaEventCreate(&a), "event");
  API_CUDA(cudaEventCreate(&b), "event");
  API_CUDA(lcp::launch_fp64_probe(out.as<double>(), blocks, threads, 64, ctx->stream), "probe");
  cudaEventRecord(a, ctx->stream);
  API_CUDA(lcp::launch_fp64_probe(out.as<double>(), blocks, threads, iters, ctx->stream), "probe");
  cudaEventRecord(b, ctx->stream);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->launches += 2;
  *tflops = 2.0 * 8.0 * (double)blocks * threads * iters / (ms * 1e-3) / 1e12;
  return LCP_OK;
}

lcp_status lcp_ctx_set_fault_test(lcp_ctx* ctx, uint32_t poll_limit, int32_t stall) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (stall < 0 || stall > 1) return fail(LCP_EINVAL, "stall is 0 or 1");
  ctx->fault_poll = poll_limit;
  ctx->fault_stall = stall;
  return LCP_OK;
}

lcp_status lcp_ctx_set_xc_arithmetic(lcp_ctx* ctx, int32_t double_float) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (double_float < 0 || double_float > 1) return fail(LCP_EINVAL, "double_float is 0 or 1");
  ctx->xc_dfl = double_float;
  return LCP_OK;
}

lcp_status lcp_bounds_check_status(lcp_ctx* ctx, int64_t* word) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!word) return fail(LCP_EINVAL, "NULL argument");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "bounds check");
  unsigned long long a = 0, b = 0;
  cudaError_t e = lcp::bounds_take_pairs(&a);
  if (e == cudaErrorNotSupported) return fail(LCP_ENOTSUP, "this library was built without bounds checks");
  API_CUDA(e, "bounds word");
  API_CUDA(lcp::bounds_take_tc(&b), "bounds word");
  *word = (int64_t)(a ? a : b);
  return LCP_OK;
}

lcp_status lcp_orbs_timings(const lcp_orbs* orbs, double* out2) {
  if (!orbs || !out2) return fail(LCP_EINVAL, "NULL argument");
  out2[0] = orbs->tab_ms;
  out2[1] = orbs->split_ms;
  return LCP_OK;
}

lcp_status lcp_device_alloc_count(int64_t* count) {
  if (!count) return fail(LCP_EINVAL, "NULL argument");
  *count = g_device_allocs.load(std::memory_order_relaxed);
  return LCP_OK;
}

lcp_status lcp_job_get_density(lcp_ctx* ctx, lcp_job* job, double* const* d) { return job_get(ctx, job, job ? job->rho : nullptr, job ? job->nn : 0, d); }
lcp_status lcp_job_get_hks(lcp_ctx* ctx, lcp_job* job, double* const* h) { return job_get(ctx, job, job ? job->hks : nullptr, job ? job->hsize : 0, h); }
lcp_status lcp_job_get_vpot(lcp_ctx* ctx, lcp_job* job, double* const* v) { return job_get(ctx, job, job ? job->vpot : nullptr, job ? job->nn : 0, v); }

}  // extern "C"

// ---------------------------------------------------------------- split-BF16 density without allocation
//
// For callers that must not allocate device memory at call time: hosts whose
// own pool allocator owns the device memory (a cudaMalloc behind its back can
// fail under that pool's reservation or fragment it), and latency-bound
// serving loops, where cudaMalloc/cudaFree may synchronise the whole device
// and stall the other streams in flight.  The scratch of the split-BF16
// density (the symmetrised fixed-point D blocks, the D scale, the |D| maximum
// and the error word) lives in the fixed array below instead of in context
// workspaces.  Its limit: 16 MiB, which holds the D blocks of up to
// kNoAllocMaxPairs neighbour pairs (1.5 KB each).  The array exists once per
// device that loads this library and is held until the process exits.

namespace {

constexpr size_t kNoAllocBytes = size_t(16) << 20;
constexpr size_t kNoAllocHeader = 256;  // [0,16) D scale, [16,24) |D| max bits, [24,28) error word
constexpr size_t kNoAllocPairBytes = 768 * sizeof(uint16_t);
constexpr int64_t kNoAllocMaxPairs = (int64_t)((kNoAllocBytes - kNoAllocHeader) / kNoAllocPairBytes) - 1;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch on the context's device (host code
// must not pass the symbol itself to a kernel).  Looked up by the context's
// first call and kept in the context, so a context made after the device's
// primary context was torn down and made again looks it up afresh.
lcp_status noalloc_scratch(lcp_ctx* ctx, unsigned char** out) {
  if (!ctx->noalloc_scratch) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
    ctx->noalloc_scratch = p;
  }
  *out = static_cast<unsigned char*>(ctx->noalloc_scratch);
  return LCP_OK;
}

}  // namespace

extern "C" {

lcp_status lcp_set_density_grid_noalloc(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs,
                                        int32_t spinpol, const double* const* dm_dev,
                                        double* const* density_grid_dev) {
  lcp_status s = check_ctx(ctx);  // makes the context's device current
  if (s) return s;
  if ((s = check_pair(ucell, orbs))) return s;
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol.");
  if (!dm_dev || !density_grid_dev) return fail(LCP_EINVAL, "NULL argument");
  const int ns = channels(spinpol);
  for (int c = 0; c < ns; ++c)
    if (!dm_dev[c] || !density_grid_dev[c]) return fail(LCP_EINVAL, "NULL channel");
  const lcp::UCell& u = ucell->u;
  if ((int64_t)u.nloop > kNoAllocMaxPairs)
    return fail(LCP_EINVAL, "the no-allocation density holds the D blocks of at most " +
                                std::to_string(kNoAllocMaxPairs) + " neighbour pairs (16 MiB); this cell has " +
                                std::to_string(u.nloop));
  if (!orbs->bricks_ready)
    return fail(LCP_ESTATE,
                "the split-BF16 tables of these orbitals are not built; one allocating split-BF16 call "
                "(lcp_set_density_grid or lcp_calc_matrix_elements at LCP_PREC_BF16X3) builds them");
  const int64_t nsub = orbs->bricks.nsub;  // == Nloop unless atoms have more than 16 orbitals
  if (nsub > kNoAllocMaxPairs)
    return fail(LCP_EINVAL, "the no-allocation density holds at most " + std::to_string(kNoAllocMaxPairs) +
                                " D blocks (16 MiB); this cell has " + std::to_string(nsub) +
                                " (16-orbital sub-blocks of its neighbour pairs)");
  unsigned char* base = nullptr;
  if ((s = noalloc_scratch(ctx, &base))) return s;
  double* dscale = reinterpret_cast<double*>(base);
  unsigned long long* dmax = reinterpret_cast<unsigned long long*>(base + 16);
  int* status = reinterpret_cast<int*>(base + 24);
  __nv_bfloat16* dsym = reinterpret_cast<__nv_bfloat16*>(base + kNoAllocHeader);
  const lcp_orbs* o = orbs;
  API_CUDA(cudaMemsetAsync(status, 0, sizeof(int), ctx->stream), "memset");
  for (int c = 0; c < ns; ++c) {
    API_CUDA(lcp::launch_absmax_scale(dm_dev[c], u.total_hsize, 2.0, dmax, dscale, ctx->stream), "dm scale");
    API_CUDA(lcp::launch_dsym(nsub, o->b_subpair.as<int32_t>(), o->b_subchunks.as<int32_t>(), o->o_atom.as<int32_t>(),
                              o->o_jatom.as<int32_t>(), o->o_boff.as<int64_t>(), o->o_partner.as<int32_t>(),
                              o->geom.numorbs, dm_dev[c], dscale, dsym, ctx->stream),
             "dsym");
    API_CUDA(lcp::launch_density_tc(o->bgeom, o->b_tab.as<__nv_bfloat16>(), o->phi_scale, dsym, dscale, (int)nsub,
                                    density_grid_dev[c], status, ctx->stream),
             "density_tc");
    ctx->launches += 4;
  }
  int st = 0;
  API_CUDA(cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "density");
  if (st) return fail(st, "a device wait timed out (tensor-core completion)");
  return LCP_OK;
}

}  // extern "C"
