// Batched SCF grid step: the device-resident jobs of many cells stepped
// together.  Every stage runs once for all cells:
//
//   - the split-D blocks, their per-cell fixed-point scales, the density and
//     the grid matrix elements each take one launch over the bricks (or
//     blocks) of every cell.  The tensor-core kernels are persistent, with one
//     CTA per SM walking a brick list that mixes the cells, heaviest bricks
//     first;
//   - Poisson runs the hand-written FFT solve once per grid shape over all of
//     that shape's cells (one block row per cell), in double-float with the
//     FP64 scaling, over contiguous per-shape buffers;
//   - the pointwise grid kernels and the FP64 reductions run over tiles of
//     every cell.  Their partition per cell is the one of a single-cell step,
//     so a cell's energy sums are the same bits as when its job steps alone.
//
// The matrix-element pass keeps one FP32 partial block per (brick, image
// pair) until its reduction; under a byte budget for those blocks the cells
// are taken in waves (consecutive cells whose blocks fit), one persistent
// launch and one reduction per wave over a shared scratch area.
//
// The whole step is recorded once as a CUDA graph and replayed.
// Everything a step touches is allocated at creation; results land in the
// jobs' own buffers (density, potential, H, energies).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <tuple>
#include <vector>

#include "lcp_api_state.h"

namespace {

struct ShapeGroup {
  int32_t ng[3];
  std::vector<int> cells;  // batch cell indices, in order
  int64_t nn = 0, nspec = 0;
  FftPlans* plan = nullptr;            // radices and roots of unity (the batch's plan cache)
  int64_t real_off = 0, spec_off = 0;  // its count * nn source doubles and count * nspec complex, in grid_pool
  int64_t cells_off = 0;               // its cells (GridCell) in fft_cells, in slot order
};

int64_t spec_len(const int32_t* ng) { return (int64_t)ng[0] * ng[1] * (ng[2] / 2 + 1); }

// A table of a batch: a place in the batch's table buffer.
struct TabRef {
  void* p = nullptr;
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// The host side of an assembly's tables: each vector at a 256-byte aligned
// offset of one byte image, bound to its TabRef once the device buffer exists.
struct Stage {
  std::vector<char> bytes;
  std::vector<std::pair<TabRef*, size_t>> refs;
  template <class T>
  void add(TabRef& r, const std::vector<T>& v) {
    const size_t off = (bytes.size() + 255) & ~size_t(255);
    bytes.resize(off + std::max<size_t>(v.size(), 1) * sizeof(T));
    if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
    refs.emplace_back(&r, off);
  }
};

// Cells [c0, c1) of the matrix-element pass that share the scratch area.
struct Wave {
  int c0 = 0, c1 = 0;
  int64_t nbricks = 0, brick_off = 0;  // its brick list in hbrick_*
  int64_t nsb = 0;                     // H sub-blocks of its cells
  int64_t order_off = 0;               // its reduction order in wred_order
};

}  // namespace

struct lcp_batch {
  int device = 0;
  int32_t spinpol = LCP_SPIN_OFF, xc = LCP_XC_LDA, nspin = 1, ncells = 0;
  std::vector<lcp_job*> jobs;
  std::vector<ShapeGroup> groups;
  std::map<std::tuple<int, int, int>, std::unique_ptr<FftPlans>> plan_cache;
  DBuf grid_pool;
  TabRef fft_cells;
  // device tables (per spin channel where the pointers differ)
  TabRef tc_cells[2], brick_cell, brick_local;
  std::vector<Wave> waves;
  TabRef hbrick_cell, hbrick_local, wred_start;  // per-wave brick lists and reduction starts
  TabRef wred_order;                             // per wave: its sub-blocks, longest first
  TabRef dsym_cells[2], dsym_start, abs_start;
  TabRef red_cells[2];
  TabRef grid_cells, pt_start, sp_start, h_start;
  // every table above lives in `tables`, uploaded from one pinned staging
  // buffer by one asynchronous copy per assembly
  DBuf tables;
  char* stage_host = nullptr;
  size_t stage_cap = 0;
  // workspaces
  DBuf dsym, dscale, dtmp, vw, vscale, hscratch, status;
  int64_t nbricks = 0, dsym_blocks = 0, abs_total = 0, nsb = 0, pt_tiles = 0, sp_tiles = 0, h_tiles = 0;
  int64_t kernels_per_step = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~lcp_batch() {
    cudaSetDevice(device);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (stage_host) cudaFreeHost(stage_host);
  }
};

namespace {


std::vector<int64_t> prefix(const std::vector<int64_t>& counts) {
  std::vector<int64_t> s(counts.size() + 1, 0);
  for (size_t i = 0; i < counts.size(); ++i) s[i + 1] = s[i] + counts[i];
  return s;
}

// Records one batched step on stream st (with events ev[0..6] at the stage
// boundaries when ev is given).
lcp_status record_step(lcp_batch* b, cudaStream_t st, cudaEvent_t* ev = nullptr) {
  auto mark = [&](int k) {
    if (ev) cudaEventRecord(ev[k], st);
  };
  const int32_t nc = b->ncells;
  lcp::TcBatch tb{};
  tb.nbricks = b->nbricks;
  tb.ncells = nc;
  tb.brick_cell = b->brick_cell.as<int32_t>();
  tb.brick_local = b->brick_local.as<int64_t>();
  const lcp::TcCell none{};
  const int64_t* wstart = b->wred_start.as<int64_t>();
  lcp::GridBatch pts{nc, b->grid_cells.as<lcp::GridCell>(), b->pt_start.as<int64_t>(), b->pt_tiles};
  lcp::GridBatch sps{nc, b->grid_cells.as<lcp::GridCell>(), b->sp_start.as<int64_t>(), b->sp_tiles};
  lcp::GridBatch hts{nc, b->grid_cells.as<lcp::GridCell>(), b->h_start.as<int64_t>(), b->h_tiles};
  lcp::GridBatch per{nc, b->grid_cells.as<lcp::GridCell>(), nullptr, nc};
  const lcp::GridCell gnone{};
  int* status = b->status.as<int>();
  // 1. density, per channel: D scales, split D blocks, the tensor-core pass
  mark(0);
  for (int c = 0; c < b->nspin; ++c) {
    const lcp::DsymCell* dc = b->dsym_cells[c].as<lcp::DsymCell>();
    // |D + D'^T| <= 2 max|D|: the fixed-point scale of the symmetrised blocks
    API_CUDA(lcp::launch_absmax_scale_batch(nc, dc, b->abs_start.as<int64_t>(), b->abs_total, 2.0,
                                            b->dtmp.as<unsigned long long>(), b->dscale.as<double>(), st),
             "batch dm scale");
    API_CUDA(lcp::launch_dsym_batch(nc, dc, b->dsym_start.as<int64_t>(), b->dsym_blocks, st), "batch dsym");
    tb.cells = b->tc_cells[c].as<lcp::TcCell>();
    API_CUDA(lcp::launch_density_tc_batch(none, tb, status, st), "batch density");
  }
  // 2. Poisson: sources, forward transforms per shape, 4 pi / G^2, inverse
  mark(1);
  for (const ShapeGroup& g : b->groups)
    API_CUDA(lcp::launch_poisson_fft(g.plan->geom, false, b->spinpol, gnone,
                                     b->fft_cells.as<lcp::GridCell>() + g.cells_off, (int)g.cells.size(), st),
             "batch poisson");
  // 3./4. xc + potential + energy partials, then the per-cell sums
  mark(2);
  if (b->xc == LCP_XC_GGA_PBE)
    API_CUDA(lcp::launch_gga_g(b->spinpol, gnone, pts, true, true, st), "batch gga");
  else
    API_CUDA(lcp::launch_xc_vpot_energy_g(b->xc, b->spinpol, gnone, pts, true, st), "batch xc");
  mark(3);
  API_CUDA(lcp::launch_grid_sums_g(gnone, per, st), "batch sums");
  mark(4);
  // 5. grid matrix elements, per channel and wave
  for (int c = 0; c < b->nspin; ++c)
    for (size_t w = 0; w < b->waves.size(); ++w) {
      const Wave& wv = b->waves[w];
      lcp::TcBatch hb{};
      hb.nbricks = wv.nbricks;
      hb.ncells = nc;
      hb.cells = b->tc_cells[c].as<lcp::TcCell>();
      hb.brick_cell = b->hbrick_cell.as<int32_t>() + wv.brick_off;
      hb.brick_local = b->hbrick_local.as<int64_t>() + wv.brick_off;
      API_CUDA(lcp::launch_hamiltonian_tc_batch(none, hb, status, st), "batch hamiltonian");
      API_CUDA(lcp::launch_h_reduce_batch(wv.c1 - wv.c0, b->red_cells[c].as<lcp::RedCell>() + wv.c0,
                                          wstart + wv.c0 + (int64_t)w, b->wred_order.as<int64_t>() + wv.order_off,
                                          wv.nsb, st),
               "batch h_reduce");
    }
  // 6. <D,H> and the energies of every cell
  mark(5);
  API_CUDA(lcp::launch_dot_energy_g(b->spinpol, b->nspin, gnone, hts, per, st), "batch dot");
  mark(6);
  return LCP_OK;
}

}  // namespace

// Fills batch b (new or used before) for these jobs: validation, shape groups,
// brick lists, waves and every device table.  Device buffers only grow, and
// FFT plans are kept per grid shape, so re-assembling a batch over another
// set of jobs of at most the same sizes allocates nothing.  The tables go up
// as one asynchronous copy on ctx's stream from pinned staging, which the
// caller must not let the next assembly of the same batch overwrite before
// the stream has passed it (a step on that stream, then a wait).  The jobs'
// split-BF16 tables are built on ctx's stream when missing.
lcp_status batch_assemble(lcp_ctx* ctx, lcp_batch* b, int32_t njobs, lcp_job* const* jobs, int64_t scratch_bytes) {
  lcp_status s = LCP_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->jobs.clear();
  b->groups.clear();
  b->waves.clear();
  b->ncells = njobs;
  Stage stage;
  for (int k = 0; k < njobs; ++k) {
    lcp_job* j = jobs[k];
    if (!j) return fail(LCP_EINVAL, "lcp_batch_create: NULL job");
    if (j->spinpol == LCP_SPIN_NC) return fail(LCP_ENOTSUP, "the batched step supports SpinPol off/on");
    if (k == 0) {
      b->spinpol = j->spinpol;
      b->xc = j->xc;
      b->nspin = j->nspin;
    } else if (j->spinpol != b->spinpol || j->xc != b->xc) {
      return fail(LCP_EINVAL, "lcp_batch_create: every job of a batch has the same SpinPol and xc");
    }
    if (j->orbs->device != ctx->device) return fail(LCP_EINVAL, "lcp_batch_create: job on another device");
    for (int q = 0; q < k; ++q)
      if (jobs[q] == j) return fail(LCP_EINVAL, "lcp_batch_create: a job appears twice");
    if ((s = ensure_bricks(ctx, const_cast<lcp_orbs*>(j->orbs)))) return s;
    b->jobs.push_back(j);
  }
  const int nc = njobs, ns = b->nspin;

  // shape groups (first appearance order) and each cell's place in its group
  std::map<std::tuple<int, int, int>, int> gidx;
  std::vector<int> cell_group(nc), cell_slot(nc);
  for (int k = 0; k < nc; ++k) {
    const int32_t* ng = b->jobs[k]->ucell->u.ngrid;
    auto key = std::make_tuple((int)ng[0], (int)ng[1], (int)ng[2]);
    auto it = gidx.find(key);
    if (it == gidx.end()) {
      it = gidx.emplace(key, (int)b->groups.size()).first;
      ShapeGroup g;
      for (int d = 0; d < 3; ++d) g.ng[d] = ng[d];
      g.nn = (int64_t)ng[0] * ng[1] * ng[2];
      g.nspec = spec_len(ng);
      auto pc = b->plan_cache.find(key);
      if (pc == b->plan_cache.end()) {
        std::unique_ptr<FftPlans> p(new FftPlans());
        if ((s = make_fft_plan(ng, p.get()))) return s;
        pc = b->plan_cache.emplace(key, std::move(p)).first;
      }
      g.plan = pc->second.get();
      b->groups.push_back(g);
    }
    ShapeGroup& g = b->groups[it->second];
    cell_group[k] = it->second;
    cell_slot[k] = (int)g.cells.size();
    g.cells.push_back(k);
  }
  // the per-shape source and spectrum buffers, carved from one pool
  {
    int64_t off = 0, coff = 0;
    for (ShapeGroup& g : b->groups) {
      const int64_t cnt = (int64_t)g.cells.size();
      g.real_off = off;
      off += cnt * g.nn;
      g.spec_off = off;
      off += cnt * g.nspec * 2;
      g.cells_off = coff;
      coff += cnt;
    }
    API_CUDA(b->grid_pool.ensure((size_t)std::max<int64_t>(off, 1) * sizeof(double)), "batch grid alloc");
  }

  // per-cell sizes and workspace offsets
  std::vector<int64_t> nbr(nc), nsub1(nc), nslot(nc), nsbc(nc), ptt(nc), spt(nc), ht(nc), abt(nc);
  for (int k = 0; k < nc; ++k) {
    const lcp_job* j = b->jobs[k];
    const lcp::Bricks& br = j->orbs->bricks;
    nbr[k] = br.nbricks;
    nsub1[k] = br.nsub + 1;
    nslot[k] = br.slot_base.back();
    nsbc[k] = (int64_t)br.sb_fold.size();
    ptt[k] = lcp::red_tiles(j->nn);
    spt[k] = lcp::red_tiles(spec_len(j->ucell->u.ngrid));
    ht[k] = lcp::red_tiles(j->hsize);
    abt[k] = lcp::abs_tiles(j->hsize);
  }
  const auto brick_off = prefix(nbr), dsym_off = prefix(nsub1), sb_off = prefix(nsbc);
  const auto pt_off = prefix(ptt), sp_off = prefix(spt), h_off = prefix(ht), ab_off = prefix(abt);
  b->nbricks = brick_off[nc];
  b->dsym_blocks = dsym_off[nc];
  b->nsb = sb_off[nc];
  b->pt_tiles = pt_off[nc];
  b->sp_tiles = sp_off[nc];
  b->h_tiles = h_off[nc];
  b->abs_total = ab_off[nc];
  API_CUDA(b->dsym.ensure((size_t)std::max<int64_t>(b->dsym_blocks, 1) * 768 * 2), "batch dsym alloc");
  API_CUDA(b->dscale.ensure((size_t)nc * 2 * sizeof(double)), "alloc");
  API_CUDA(b->dtmp.ensure((size_t)nc * sizeof(unsigned long long)), "alloc");
  API_CUDA(b->vw.ensure((size_t)std::max<int64_t>(b->nbricks, 1) * 128 * sizeof(float2)), "batch V weight alloc");
  API_CUDA(b->vscale.ensure((size_t)std::max<int64_t>(b->nbricks, 1) * sizeof(float)), "alloc");
  // waves of consecutive cells whose partial H blocks fit the budget
  std::vector<int64_t> wslot(nc);  // first scratch slot of each cell within its wave
  {
    const int64_t cap = scratch_bytes > 0 ? scratch_bytes / 1024 : INT64_MAX;  // 1 KB per partial block
    Wave cur;
    int64_t used = 0, most = 0;
    for (int k = 0; k < nc; ++k) {
      if (k > cur.c0 && used + nslot[k] > cap) {
        cur.c1 = k;
        b->waves.push_back(cur);
        cur = Wave();
        cur.c0 = k;
        used = 0;
      }
      wslot[k] = used;
      used += nslot[k];
      most = std::max(most, used);
    }
    cur.c1 = nc;
    b->waves.push_back(cur);
    API_CUDA(b->hscratch.ensure((size_t)std::max<int64_t>(most, 1) * 256 * sizeof(float)), "batch H scratch");
  }
  API_CUDA(b->status.ensure(sizeof(int)), "alloc");
  API_CUDA(cudaMemsetAsync(b->status.p, 0, sizeof(int), ctx->stream), "memset");

  // brick list: every cell's bricks, heaviest first (the persistent CTAs take
  // bricks k, k + grid, ... so a descending order balances them); the order
  // changes no result -- each brick writes its own points and partial blocks
  {
    // heaviest first = most images first (the cost m^2 + 8m grows with m):
    // a stable counting sort by m, so ties keep (cell, brick) order -- the
    // order of a stable comparison sort, in linear time
    auto sorted_bricks = [&](int c0, int c1, std::vector<int32_t>& bc, std::vector<int64_t>& bl) {
      int64_t maxm = 0, n = 0;
      for (int k = c0; k < c1; ++k) {
        const lcp::Bricks& br = b->jobs[k]->orbs->bricks;
        for (int64_t hb = 0; hb < br.nbricks; ++hb) maxm = std::max(maxm, br.img_off[hb + 1] - br.img_off[hb]);
        n += br.nbricks;
      }
      std::vector<int64_t> pos(maxm + 1, 0);
      for (int k = c0; k < c1; ++k) {
        const lcp::Bricks& br = b->jobs[k]->orbs->bricks;
        for (int64_t hb = 0; hb < br.nbricks; ++hb) ++pos[br.img_off[hb + 1] - br.img_off[hb]];
      }
      int64_t acc = (int64_t)bc.size();
      for (int64_t m = maxm; m >= 0; --m) {
        const int64_t c = pos[m];
        pos[m] = acc;
        acc += c;
      }
      bc.resize(bc.size() + n);
      bl.resize(bl.size() + n);
      for (int k = c0; k < c1; ++k) {
        const lcp::Bricks& br = b->jobs[k]->orbs->bricks;
        for (int64_t hb = 0; hb < br.nbricks; ++hb) {
          const int64_t i = pos[br.img_off[hb + 1] - br.img_off[hb]]++;
          bc[i] = (int32_t)k;
          bl[i] = hb;
        }
      }
    };
    std::vector<int32_t> bc, hbc;
    std::vector<int64_t> bl, hbl, wst, word;
    sorted_bricks(0, nc, bc, bl);
    for (Wave& w : b->waves) {
      w.brick_off = (int64_t)hbc.size();
      if (w.c0 == 0 && w.c1 == nc) {  // one wave: the same list
        hbc.insert(hbc.end(), bc.begin(), bc.end());
        hbl.insert(hbl.end(), bl.begin(), bl.end());
      } else {
        sorted_bricks(w.c0, w.c1, hbc, hbl);
      }
      w.nbricks = (int64_t)hbc.size() - w.brick_off;
      // reduction starts of the wave's cells, rebased: wst[c0 + w .. c1 + w]
      int64_t acc = 0;
      for (int k = w.c0; k < w.c1; ++k) {
        wst.push_back(acc);
        acc += nsbc[k];
      }
      wst.push_back(acc);
      w.nsb = acc;
      // the wave's sub-blocks longest first (stable): the reduction of a long
      // one started late would run alone at the end of the launch; each
      // sub-block's own sum is unchanged
      w.order_off = (int64_t)word.size();
      // (a stable counting sort by the number of partials)
      int64_t maxl = 0;
      for (int k = w.c0; k < w.c1; ++k) {
        const std::vector<int64_t>& ro = b->jobs[k]->orbs->bricks.red_off;
        for (int64_t u = 0; u < nsbc[k]; ++u) maxl = std::max(maxl, ro[u + 1] - ro[u]);
      }
      std::vector<int64_t> pos(maxl + 1, 0);
      for (int k = w.c0; k < w.c1; ++k) {
        const std::vector<int64_t>& ro = b->jobs[k]->orbs->bricks.red_off;
        for (int64_t u = 0; u < nsbc[k]; ++u) ++pos[ro[u + 1] - ro[u]];
      }
      int64_t at = (int64_t)word.size();
      for (int64_t l = maxl; l >= 0; --l) {
        const int64_t c = pos[l];
        pos[l] = at;
        at += c;
      }
      word.resize(word.size() + acc);
      int64_t g = 0;
      for (int k = w.c0; k < w.c1; ++k) {
        const std::vector<int64_t>& ro = b->jobs[k]->orbs->bricks.red_off;
        for (int64_t u = 0; u < nsbc[k]; ++u, ++g) word[pos[ro[u + 1] - ro[u]]++] = g;
      }
    }
    stage.add(b->brick_cell, bc);
    stage.add(b->brick_local, bl);
    stage.add(b->hbrick_cell, hbc);
    stage.add(b->hbrick_local, hbl);
    stage.add(b->wred_start, wst);
    stage.add(b->wred_order, word);
  }

  // per-cell tables
  std::vector<lcp::GridCell> gcs(nc);
  for (int k = 0; k < nc; ++k) {
    lcp_job* j = b->jobs[k];
    const ShapeGroup& g = b->groups[cell_group[k]];
    lcp::GridCell c = job_grid_cell(j);
    c.real = b->grid_pool.as<double>() + g.real_off + (int64_t)cell_slot[k] * g.nn;
    c.spec = b->grid_pool.as<double>() + g.spec_off + (int64_t)cell_slot[k] * g.nspec * 2;
    c.dvh = c.real;  // the inverse transform writes back over the source
    gcs[k] = c;
  }
  stage.add(b->grid_cells, gcs);
  {
    std::vector<lcp::GridCell> fc;
    for (const ShapeGroup& g : b->groups)
      for (int k : g.cells) fc.push_back(gcs[k]);
    stage.add(b->fft_cells, fc);
  }
  for (int ch = 0; ch < ns; ++ch) {
    std::vector<lcp::TcCell> tcs(nc);
    std::vector<lcp::DsymCell> dcs(nc);
    std::vector<lcp::RedCell> rcs(nc);
    for (int k = 0; k < nc; ++k) {
      lcp_job* j = b->jobs[k];
      const lcp_orbs* o = j->orbs;
      const lcp::UCell& u = j->ucell->u;
      __nv_bfloat16* dsym = b->dsym.as<__nv_bfloat16>() + dsym_off[k] * 768;
      const double* dscale = b->dscale.as<double>() + 2 * k;
      float* scratch = b->hscratch.as<float>() + wslot[k] * 256;
      lcp::TcCell t = lcp::tc_cell_of(o->bgeom, o->b_tab.as<__nv_bfloat16>());
      t.phi_scale = o->phi_scale;
      t.dsym = dsym;
      t.zero_pair = o->bricks.nsub;
      t.dscale = dscale;
      t.rho = j->rho[ch].as<double>();
      t.tab_slot = o->b_tabslot.as<int32_t>();
      t.slot_base = o->b_slotbase.as<int64_t>();
      t.vpot = j->vpot[ch].as<double>();
      t.vw = b->vw.as<float2>() + brick_off[k] * 128;
      t.vscale = b->vscale.as<float>() + brick_off[k];
      t.scratch = scratch;
      tcs[k] = t;
      lcp::DsymCell d{};
      d.nsub = o->bricks.nsub;
      d.hsize = j->hsize;
      d.scale = dscale;
      d.sub_pair = o->b_subpair.as<int32_t>();
      d.sub_chunks = o->b_subchunks.as<int32_t>();
      d.pair_atom = o->o_atom.as<int32_t>();
      d.pair_jatom = o->o_jatom.as<int32_t>();
      d.boff = o->o_boff.as<int64_t>();
      d.partner = o->o_partner.as<int32_t>();
      d.numorbs = o->geom.numorbs;
      d.dm = j->dm[ch].as<double>();
      d.out = dsym;
      dcs[k] = d;
      lcp::RedCell r{};
      r.red_off = o->b_redoff.as<int64_t>();
      r.red_slot = o->b_redslot.as<int64_t>();
      r.sb_fold = o->b_sbfold.as<int32_t>();
      r.sb_chunks = o->b_sbchunks.as<int32_t>();
      r.scratch = scratch;
      r.pr = o->pairs;
      r.numorbs = o->geom.numorbs;
      r.dv = u.gridvol;
      r.H = j->hks[ch].as<double>();
      rcs[k] = r;
    }
    stage.add(b->tc_cells[ch], tcs);
    stage.add(b->dsym_cells[ch], dcs);
    stage.add(b->red_cells[ch], rcs);
  }
  stage.add(b->dsym_start, dsym_off);
  stage.add(b->abs_start, ab_off);
  stage.add(b->pt_start, pt_off);
  stage.add(b->sp_start, sp_off);
  stage.add(b->h_start, h_off);
  // our kernels per step: per channel absmax + pow2 + dsym + density, per
  // channel and wave vweight + H + reduce; the five FFT passes per grid
  // shape; once xc, sums, dot, dot-finish (GGA-PBE: xc is two passes)
  b->kernels_per_step = 4 * ns + 3 * ns * (int64_t)b->waves.size() + 4 + 5 * (int64_t)b->groups.size() +
                        (b->xc == LCP_XC_GGA_PBE ? 1 : 0);
  // one copy of every table: pinned staging (grown when needed), one device buffer
  const size_t nbytes = std::max<size_t>(stage.bytes.size(), 1);
  API_CUDA(b->tables.ensure(nbytes), "batch tables alloc");
  if (nbytes > b->stage_cap) {
    if (b->stage_host) cudaFreeHost(b->stage_host);
    b->stage_host = nullptr;
    b->stage_cap = 0;
    API_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&b->stage_host), nbytes, cudaHostAllocDefault),
             "batch staging alloc");
    b->stage_cap = nbytes;
  }
  std::memcpy(b->stage_host, stage.bytes.data(), stage.bytes.size());
  API_CUDA(cudaMemcpyAsync(b->tables.p, b->stage_host, stage.bytes.size(), cudaMemcpyHostToDevice, ctx->stream),
           "batch tables upload");
  for (auto& r : stage.refs) r.first->p = static_cast<char*>(b->tables.p) + r.second;
  return LCP_OK;
}

lcp_batch* batch_new(int device) {
  lcp_batch* b = new lcp_batch();
  b->device = device;
  return b;
}

// Records one eager step of an assembled batch on `st` (no graph).
lcp_status batch_record(lcp_batch* b, cudaStream_t st) { return record_step(b, st); }

// The device status word of the batch's tensor-core kernels (for a caller
// that synchronises the stream itself); clears it.
lcp_status batch_status(lcp_batch* b, cudaStream_t st) {
  int v = 0;
  API_CUDA(cudaMemcpyAsync(&v, b->status.p, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
  API_CUDA(cudaStreamSynchronize(st), "status");
  if (v) {
    cudaMemsetAsync(b->status.p, 0, sizeof(int), st);
    return fail(v, "a device wait timed out (batched tensor-core step)");
  }
  return LCP_OK;
}

extern "C" {

lcp_status lcp_batch_create(lcp_ctx* ctx, int32_t njobs, lcp_job* const* jobs, int64_t scratch_bytes,
                            lcp_batch** out) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!jobs || !out || njobs <= 0 || scratch_bytes < 0)
    return fail(LCP_EINVAL, "lcp_batch_create: NULL argument, no jobs or a negative budget");
  *out = nullptr;
  if (ctx->precision != LCP_PREC_BF16X3)
    return fail(LCP_ENOTSUP, "the batched step runs the split-BF16 contractions (precision bf16x3)");
  std::unique_ptr<lcp_batch> b(batch_new(ctx->device));
  if ((s = batch_assemble(ctx, b.get(), njobs, jobs, scratch_bytes))) return s;
  API_CUDA(cudaDeviceSynchronize(), "batch create");
  *out = b.release();
  return LCP_OK;
}

void lcp_batch_destroy(lcp_batch* batch) { delete batch; }

lcp_status lcp_batch_step(lcp_ctx* ctx, lcp_batch* b, int32_t mode) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!b) return fail(LCP_EINVAL, "NULL batch");
  if (ctx->device != b->device) return fail(LCP_EINVAL, "batch on another device");
  if (mode == LCP_BATCH_EAGER) {
    if ((s = record_step(b, ctx->stream))) return s;
  } else if (mode == LCP_BATCH_GRAPH) {
    if (!b->exec) {
      // the first step runs eagerly (module loading, kernel attributes), the
      // capture of the second becomes the graph that every later step replays
      if ((s = record_step(b, ctx->stream))) return s;
      API_CUDA(cudaStreamSynchronize(ctx->stream), "batch warm-up");
      cudaStream_t cap = nullptr;
      API_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "capture stream");
      cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed);
      if (e == cudaSuccess) {
        lcp_status rs = record_step(b, cap);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(cap, &g);
        if (rs != LCP_OK) {
          if (g) cudaGraphDestroy(g);
          cudaStreamDestroy(cap);
          return rs;
        }
        if (e == cudaSuccess) {
          b->graph = g;
          e = cudaGraphInstantiate(&b->exec, g, 0);
        }
      }
      cudaStreamDestroy(cap);
      API_CUDA(e, "batch graph capture");
      ctx->launches += b->kernels_per_step;
      return LCP_OK;
    }
    API_CUDA(cudaGraphLaunch(b->exec, ctx->stream), "cudaGraphLaunch");
  } else {
    return fail(LCP_EINVAL, "lcp_batch_step: mode is LCP_BATCH_GRAPH or LCP_BATCH_EAGER");
  }
  ctx->launches += b->kernels_per_step;
  return LCP_OK;
}

lcp_status lcp_batch_step_timed(lcp_ctx* ctx, lcp_batch* b, double* stage_ms) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!b || !stage_ms) return fail(LCP_EINVAL, "NULL argument");
  if (ctx->device != b->device) return fail(LCP_EINVAL, "batch on another device");
  cudaEvent_t ev[7];
  for (int k = 0; k < 7; ++k) API_CUDA(cudaEventCreate(&ev[k]), "cudaEventCreate");
  s = record_step(b, ctx->stream, ev);
  if (s == LCP_OK) {
    ctx->launches += b->kernels_per_step;
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

lcp_status lcp_batch_check_status(lcp_ctx* ctx, lcp_batch* b) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!b) return fail(LCP_EINVAL, "NULL batch");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "batch status");
  int st = 0;
  API_CUDA(cudaMemcpy(&st, b->status.p, sizeof(int), cudaMemcpyDeviceToHost), "status");
  if (st) {
    cudaMemset(b->status.p, 0, sizeof(int));
    return fail(st, "a device wait timed out (batched tensor-core step)");
  }
  return LCP_OK;
}

lcp_status lcp_batch_energies(lcp_ctx* ctx, lcp_batch* b, double* out) {
  lcp_status s = lcp_batch_check_status(ctx, b);
  if (s) return s;
  if (!out) return fail(LCP_EINVAL, "NULL argument");
  for (int k = 0; k < b->ncells; ++k)
    API_CUDA(cudaMemcpyAsync(out + 5 * k, b->jobs[k]->scal.as<double>() + 8, 5 * sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->stream),
             "D2H");
  API_CUDA(cudaStreamSynchronize(ctx->stream), "batch energies");
  return LCP_OK;
}

lcp_status lcp_batch_info(const lcp_batch* b, int64_t* out8) {
  if (!b || !out8) return fail(LCP_EINVAL, "NULL argument");
  out8[0] = b->ncells;
  out8[1] = (int64_t)b->groups.size();
  out8[2] = b->nbricks;
  out8[3] = b->kernels_per_step;
  int64_t bytes = 0;
  for (const DBuf* d : {&b->dsym, &b->vw, &b->vscale, &b->hscratch})
    bytes += (int64_t)d->bytes;
  bytes += (int64_t)b->grid_pool.bytes;
  for (const auto& kv : b->plan_cache) bytes += (int64_t)kv.second->roots.bytes;
  out8[4] = bytes;
  out8[5] = b->exec ? 1 : 0;
  out8[6] = b->nsb;
  out8[7] = (int64_t)b->waves.size();
  return LCP_OK;
}

}  // extern "C"
