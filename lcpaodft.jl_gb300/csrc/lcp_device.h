// Device-side structures and kernel launchers shared by the .cu files.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <algorithm>
#include <vector>

#include "lcpgrid.h"

namespace lcp {

#define LCP_CUDA_TRY(expr)                                                   \
  do {                                                                       \
    cudaError_t _e = (expr);                                                 \
    if (_e != cudaSuccess) return _e;                                        \
  } while (0)

constexpr int kMaxL = 3;

// Raises kernel's dynamic shared-memory limit on the current device to at
// least `bytes` (never lowers it).  The limit is one attribute of the kernel
// shared by every host thread that launches it, so a launcher whose size
// varies between calls must not set it to its own size: another thread's
// larger launch in between would fail.
cudaError_t raise_smem_limit(const void* kernel, size_t bytes);
template <class F>
cudaError_t raise_smem(F* kernel, size_t bytes) {
  return raise_smem_limit(reinterpret_cast<const void*>(kernel), bytes);
}

// Radial tables of one species in device memory.
struct DevSpecies {
  int32_t max_l;
  int32_t nb[4];
  int32_t nmesh;
  int32_t nrad;      // number of radial functions = sum_l nb[l]
  int32_t no;        // orbitals = sum_l nb[l]*(2l+1)
  int64_t rv_off;    // offset of RV in the packed radial array
  int64_t rwf_off;   // offset of RWF[(l,p)][mesh] in the packed radial array
  // value tables' spline, precomputed per mesh interval (append_spline_tables):
  int64_t iv_off;    // per interval m: RV[m-1], 1/(RV[m]-RV[m-1]), then per radial c0..c3
  int64_t ex_off;    // per radial: a, b, c, d of the extrapolation below RV[0]
  int64_t bk_off;    // bucket table (int32 array): first mesh index of each log2(R) bucket
  float bk_lo, bk_inv;  // bucket of R: (log2(R) - bk_lo) * bk_inv
};
constexpr int kSplineBuckets = 4096;
// Appends the per-interval cubic coefficients of the value tables'
// radial spline, the extrapolation coefficients and the interval buckets of
// one species (rv, rwf as lcp_pao) to `radial` / `buckets`; fills d's offsets.
void append_spline_tables(const double* rv, const double* rwf, int nmesh, const int* num_basis, int max_l,
                          DevSpecies& d, std::vector<double>& radial, std::vector<int32_t>& buckets);

// Geometry the kernels read (device pointers).
struct DevGeom {
  int32_t natom;
  int32_t ngrid[3];
  double glat[9];     // row d = Latvecs[d,:]/Ngrid[d]
  double origin[3];
  double gridvol;
  const double* atv;         // ncell*3
  const double* gxyz;        // natom*3
  const int32_t* spe;        // natom, 0-based species
  const int64_t* sph_off;    // natom+1, offsets into glist/clist
  const int32_t* glist;
  const int32_t* clist;
  const int64_t* phi_off;    // natom+1, offset of each atom's table (elements)
  const int32_t* numorbs;    // natom
};

// Folded pair list (one of each {(i,j,R), (j,i,-R)}) with exact lens lists.
struct DevPairs {
  int64_t nu;
  const int32_t* atom;       // nu, 0-based
  const int32_t* jatom;      // nu
  const int64_t* boff_p;     // block offset of the kept orientation
  const int64_t* boff_q;     // block offset of the partner (== boff_p for self pairs)
  const int32_t* self;       // nu, 1 when the pair is its own partner
  const int64_t* lens_off;   // nu+1
  const int32_t* g1;         // index into atom's sphere list
  const int32_t* g2;         // index into jatom's sphere list
  int64_t hsize;             // Total_Hsize (DM/H blocks), for the check build
  // chunked work items over the lens lists
  int64_t nitems;
  const int64_t* item_pair;  // folded pair of each item
  const int64_t* item_start; // first lens entry
  const int32_t* item_count; // number of lens entries
};

// tabulation
// nblocks blocks of kTabBlock sphere points (block_atom / block_start); phi
// alone: the value kernel; with dphi_*: values and gradient tables.  max_no:
// the largest orbital count of the species (shared-memory staging).
constexpr int kTabBlock = 128;
cudaError_t launch_tabulate(const DevGeom& g, const DevSpecies* dspe, const double* radial, const int32_t* buckets,
                            int64_t nblocks, const int32_t* block_atom, const int64_t* block_start,
                            double* phi, double* dphi_x, double* dphi_y, double* dphi_z, int max_no,
                            cudaStream_t st);
cudaError_t launch_convert_f32(const double* src, float* dst, int64_t n, cudaStream_t st);

// The check build's first bounds violation of the pair kernels and of the
// tensor-core kernels (0: none), read and cleared; cudaErrorNotSupported in
// the normal build.
cudaError_t bounds_take_pairs(unsigned long long* word);
cudaError_t bounds_take_tc(unsigned long long* word);

// exact-lens pair contractions
cudaError_t launch_density_pairs(int prec, const DevGeom& g, const DevPairs& pr, int nspin,
                                 const double* phi64, const float* phi32, const double* const* dm,
                                 double* const* rho, int max_no, cudaStream_t st);
cudaError_t launch_hamiltonian_pairs(int prec, const DevGeom& g, const DevPairs& pr, int nch,
                                     const double* phi64, const float* phi32,
                                     const double* const* vpot, double* const* hks, int max_no,
                                     cudaStream_t st);

// grid force term (FP64): per work item the six sums of both orientations
// (partials: 6 * nitems doubles), then per atom the sum of its entries
// (item * 2 + orientation) times gridvol into force[natom][3]
cudaError_t launch_force3_pairs(const DevGeom& g, const DevPairs& pr, int nch, const double* phi,
                                const double* const* dphi, const double* const* vpot, const double* const* dm,
                                const double* coef, double* partials, int max_no, cudaStream_t st);
cudaError_t launch_force3_reduce(int natom, const int64_t* off, const int64_t* code, const double* partials,
                                 double gridvol, double* force, cudaStream_t st);

// grid kernels
cudaError_t launch_poisson_prep(int spinpol, int64_t nn, const double* rho0, const double* rho1,
                                const double* aden, double* out, cudaStream_t st);
cudaError_t launch_poisson_scale(const int32_t* ngrid, const double* recvecs, void* spectrum,
                                 cudaStream_t st);
cudaError_t launch_xc_vpot(int xc, int spinpol, int64_t nn, const double* pcc,
                           const double* const* rho, const double* dvh, const double* vna,
                           double* const* vxc_out, double* const* vpot_out, cudaStream_t st);
cudaError_t launch_vpot(int spinpol, int64_t nn, const double* dvh, const double* const* vxc,
                        const double* vna, double* const* vpot, cudaStream_t st);
// Deterministic FP64 energy sums: out[0] = sum dRho*dVH, out[1..2] = xc sums;
// partials: 3 * red_tiles(nn) doubles.
cudaError_t launch_energy_sums(int xc, int spinpol, int64_t nn, const double* aden,
                               const double* pcc, const double* const* rho, const double* dvh,
                               double* partials, double* out, cudaStream_t st);
// Reductions run over tiles of kRedTile elements, one block per tile.
constexpr int kRedTile = 1024;
__host__ __device__ inline int64_t red_tiles(int64_t n) { return n > 0 ? (n + kRedTile - 1) / kRedTile : 0; }

// One cell of a grid-step pass: its grid, the fields it reads and writes, and
// its reduction partials.  A launch covers one cell (passed by value) or a
// batch of cells (a device table); a cell's results are the same bits either
// way.
struct GridCell {
  int32_t ng[3];
  int64_t nn, hsize;
  double rv[9];          // reciprocal vectors (rows), 2*pi*inv(Latvecs')
  double gridvol;
  const double* aden;    // atomic density or nullptr
  const double* pcc;     // partial core correction or nullptr
  const double* vna;     // neutral-atom potential or nullptr
  const double* rho[4];  // [2..3]: the "nc" angles theta, phi after diagonalize_nc_density!
  double* real;          // Poisson source (nn)
  void* spec;            // its half spectrum (ng0 * ng1 * (ng2/2+1) complex)
  const double* pfac;    // tabulated Poisson factors of the half spectrum, or nullptr
  const double* dvh;     // Hartree potential (nn)
  double* vpot[4];
  const double* dm[4];
  const double* hks[4];
  double* part;          // tile partials: 3 * red_tiles(nn) and red_tiles(hsize) doubles
  double* sums;          // [0..2] grid sums, [3] sum <D,H>, [8..12] the step's energies
  // GGA-PBE only (nullptr otherwise)
  const double* dcoef;   // gradient stencil weights [3][27] (Calc_Diff_Coef)
  double* dexc;          // dE/d(grad rho) scratch: [spin][xyz][nn]
  double* dden;          // optional output: grad(rho + pcc) as [spin][xyz][nn]
};
// cells == nullptr: the single cell passed by value.  Otherwise block g of a
// tiled launch belongs to the cell c with start[c] <= g < start[c+1], and a
// per-cell launch has one block per cell.
struct GridBatch {
  int32_t ncells;
  const GridCell* cells;
  const int64_t* start;
  int64_t nblocks;
};
// Hand-written FFT Poisson solve (lcp_fft.cu): per cell, dvh = the solve of
// its source (2rho - 2rho_a "off", rho_up + rho_down - 2rho_a otherwise, or
// with spinpol < 0 the cell's real array as is), through its half-spectrum
// scratch spec and its factors pfac.  One cell by value (cells == nullptr) or
// ncells cells of one grid shape from a device table.  fp64: FP64
// transforms, else double-float transforms with the FP64 scaling.
constexpr int kFftMaxN = 1024;       // longest supported grid dimension
constexpr int kFftMaxFactors = 24;
struct FftGeom {
  int32_t n[3];
  int32_t nfac[3];
  int32_t fac[3][kFftMaxFactors];
  const void* roots64[3];  // per axis: its n roots of unity, complex double
  const void* roots32[3];  // the same as double-float: re.hi, re.lo, im.hi, im.lo
};
int fft_factor(int n, int* fac);
bool fft_supported(const int32_t* ng);
void fft_roots(int n, std::vector<double>& r64, std::vector<float>& r32);
cudaError_t launch_poisson_fft(const FftGeom& g, bool fp64, int spinpol, const GridCell& c0, const GridCell* cells,
                               int ncells, cudaStream_t st);
cudaError_t launch_poisson_prep_g(int spinpol, const GridCell& c0, const GridBatch& b, cudaStream_t st);
cudaError_t launch_poisson_scale_g(const GridCell& c0, const GridBatch& b, cudaStream_t st);
// The Poisson factors of a grid (ng0 * ng1 * (ng2/2+1) doubles), for GridCell::pfac.
cudaError_t launch_poisson_table(const int32_t* ngrid, const double* recvecs, double* out, cudaStream_t st);
// xc + potential + the energy-term tile partials in one pass (tiles of nn)
// With dvh == nullptr in the cell, the xc pass writes vxc to vpot and leaves
// the E_H1 partials zero; launch_vpot_eh_g then adds dVHart + V_na and the
// E_H1 partials (spinpol "off" or "on").
// dfl: the functional in double-float (the precision forms), else FP64.
cudaError_t launch_xc_vpot_energy_g(int xc, int spinpol, const GridCell& c0, const GridBatch& b, bool dfl,
                                    cudaStream_t st);
cudaError_t launch_xc_selftest(int xc, bool dfl, int64_t nn, const double* up, const double* dn, const double* pcc,
                               double* out, cudaStream_t st);
cudaError_t launch_vpot_eh_g(int spinpol, const GridCell& c0, const GridBatch& b, cudaStream_t st);
// GGA-PBE pass of the grid step (cells with dcoef/dexc set): gradient + PBE
// (+ energy tile partials where part is set), then, if potential, the
// divergence term and, where dvh is set, vpot = dVHart + vxc + V_na (without
// dvh, vpot receives vxc).  spinpol "off" or "on".
cudaError_t launch_gga_g(int spinpol, const GridCell& c0, const GridBatch& b, bool potential, bool dfl,
                         cudaStream_t st);
// "nc": diagonalize_nc_density! in place, (Re11, Re22, Re12, Im12) -> (Nup,
// Ndown, theta, phi), and the rotation of collinear potentials (vu, vd) into
// the four channels by the local angles; out[0..1] may be vu/vd.  sign3 is the
// sign of the third channel's tmp1 sin(theta) cos(phi): +1 for LDA/LSDA
// (src/XC/XC_Func.jl:130-142), -1 for GGA-PBE (src/XC/GGA_PBE.jl:174-192).
cudaError_t launch_nc_diagonalize(int64_t nn, double* const* rho, cudaStream_t st);
cudaError_t launch_nc_rotate(int64_t nn, const double* vu, const double* vd, const double* theta, const double* phi,
                             double sign3, double* const* out, cudaStream_t st);
// per cell: sums[0..2] from the energy partials
cudaError_t launch_grid_sums_g(const GridCell& c0, const GridBatch& b, cudaStream_t st);
// <D,H> tile partials (tiles of hsize), then per cell sums[3] and the energies
cudaError_t launch_dot_energy_g(int spinpol, int nspin, const GridCell& c0, const GridBatch& tiles,
                                const GridBatch& cells, cudaStream_t st);
cudaError_t launch_fp64_probe(double* out, int blocks, int threads, int iters, cudaStream_t st);
// Device copy of the brick tiling (see struct Bricks in lcp_internal.h).
struct TcBrickGeom {
  int64_t nbricks;
  int64_t nblocks;  // table blocks = images; brick hb's images are blocks img_off[hb] .. img_off[hb+1]-1
  int32_t bdim[3], nb[3], ngrid[3];
  int32_t npts, max_images;
  const int64_t* img_off;
  const int32_t* img_block;
  const int64_t* tab_off;
  const int32_t* tab_pair;
};
// One cell of a tensor-core launch: its brick tiling and tables, and where the
// step reads and writes.  A batch launch covers the bricks of several cells.
struct TcCell {
  int64_t nbricks, nblocks;
  int32_t bdim[3], nb[3], ngrid[3];
  int32_t npts;
  const __nv_bfloat16* tab;    // part-major split-BF16 tables of the cell
  const int64_t* img_off;      // [nbricks+1]
  const int64_t* tab_off;      // [nbricks+1]
  const int32_t* tab_pair;     // sub-pair tables (density)
  const int32_t* tab_slot;     // slot tables (matrix elements)
  const int64_t* slot_base;    // [nbricks+1]
  double phi_scale;            // S_phi of the tables
  const __nv_bfloat16* dsym;   // density: split D blocks, zero block at zero_pair
  int64_t zero_pair;
  const double* dscale;        // density: [S_D, 1/S_D] of the cell's D
  double* rho;                 // density output (one spin channel)
  const double* vpot;          // matrix elements: V (one channel)
  float2* vw;                  // [nbricks * 128] per-brick V weights (workspace)
  float* vscale;               // [nbricks]
  float* scratch;              // partial blocks, slot_base-indexed
};
// Several cells in one launch: brick k of the launch is brick brick_local[k]
// of cell brick_cell[k].  cells == nullptr: a single cell, passed by value.
struct TcBatch {
  int64_t nbricks;
  int32_t ncells;
  const TcCell* cells;
  const int32_t* brick_cell;
  const int64_t* brick_local;
};
TcCell tc_cell_of(const TcBrickGeom& bg, const __nv_bfloat16* tab);
// Batched split D blocks: cell c's sub-pairs (and its zero block) at
// start[c] .. start[c+1] of the launch's blocks.
struct DsymCell {
  int64_t nsub, hsize;
  const double* scale;  // [S_D, 1/S_D] of the cell
  const int32_t* sub_pair;
  const int32_t* sub_chunks;
  const int32_t* pair_atom;
  const int32_t* pair_jatom;
  const int64_t* boff;
  const int32_t* partner;
  const int32_t* numorbs;
  const double* dm;
  __nv_bfloat16* out;
};
cudaError_t launch_dsym_batch(int32_t ncells, const DsymCell* cells, const int64_t* start, int64_t total_blocks,
                              cudaStream_t st);
// Per-cell fixed-point scale of D: scale[2c] = power of two >= factor * max|D_c|,
// scale[2c+1] its inverse; start over abs_tiles(hsize) tiles per cell; tmp: ncells words.
int64_t abs_tiles(int64_t n);
cudaError_t launch_absmax_scale_batch(int32_t ncells, const DsymCell* cells, const int64_t* start, int64_t total_tiles,
                                      double factor, unsigned long long* tmp, double* scale, cudaStream_t st);
// Batched partial-block reduction: cell c's H sub-blocks at start[c] .. start[c+1].
struct RedCell {
  const int64_t* red_off;
  const int64_t* red_slot;
  const int32_t* sb_fold;
  const int32_t* sb_chunks;
  const float* scratch;
  DevPairs pr;
  const int32_t* numorbs;
  double dv;
  double* H;
};
cudaError_t launch_h_reduce_batch(int32_t ncells, const RedCell* cells, const int64_t* start, const int64_t* order,
                                  int64_t total, cudaStream_t st);
// poll: polls of every bounded wait before it gives up (0: 2^24); stall: for
// failure-path tests only, 1 makes one epilogue warp withhold its stage
// releases so that the kernel times out and unwinds.
cudaError_t launch_density_tc_batch(const TcCell& cell0, const TcBatch& batch, int* status, cudaStream_t st,
                                    uint32_t poll = 0, int32_t stall = 0);
// ev_begin / ev_end (optional): recorded around the tensor-core kernel itself
cudaError_t launch_hamiltonian_tc_batch(const TcCell& cell0, const TcBatch& batch, int* status, cudaStream_t st,
                                        cudaEvent_t ev_begin = nullptr, cudaEvent_t ev_end = nullptr);
cudaError_t launch_absmax_scale(const double* x, int64_t n, double factor, unsigned long long* tmp, double* scale,
                                cudaStream_t st);
// The split-BF16 tables from the FP64 tables: first_block[nimg] lists the
// first block of every atom image (its 16-orbital chunks follow it), which
// together cover all nblocks blocks; slot_point is scratch of nblocks * 128
// ints.
cudaError_t launch_brick_table(const double* phi, const int64_t* phi_off, const int32_t* numorbs,
                               const int64_t* sph_off, const int32_t* point_code, int64_t npoints,
                               const int32_t* block_atom, const int32_t* first_block, int64_t nimg,
                               int32_t* slot_point, const double* scale, __nv_bfloat16* tab, int64_t nblocks,
                               cudaStream_t st);
cudaError_t launch_dsym(int64_t nsub, const int32_t* sub_pair, const int32_t* sub_chunks, const int32_t* pair_atom,
                        const int32_t* pair_jatom, const int64_t* boff, const int32_t* partner, const int32_t* numorbs,
                        const double* dm, const double* scale, __nv_bfloat16* out, cudaStream_t st);
cudaError_t launch_density_tc(const TcBrickGeom& bg, const __nv_bfloat16* tab, double phi_scale,
                              const __nv_bfloat16* dsym, const double* dscale, int zero_pair, double* rho,
                              int* status, cudaStream_t st, uint32_t poll = 0, int32_t stall = 0);
cudaError_t launch_tc_selftest(const float* A, const float* B, float* D, int N, int K, int a_mn, int b_mn,
                               int order, int* status, cudaStream_t st);
// vw: nbricks * 128 float2 and vscale: nbricks floats of workspace (the
// per-brick V weights); scratch: the FP32 partial blocks.
cudaError_t launch_hamiltonian_tc(const TcBrickGeom& bg, const int32_t* tab_slot, const int64_t* slot_base,
                                  const __nv_bfloat16* tab, double phi_scale, const double* vpot, float2* vw,
                                  float* vscale, float* scratch, int* status, cudaStream_t st,
                                  cudaEvent_t ev_begin = nullptr, cudaEvent_t ev_end = nullptr);
cudaError_t launch_h_reduce(int64_t nsb, const int64_t* red_off, const int64_t* red_slot, const int32_t* sb_fold,
                            const int32_t* sb_chunks, const float* scratch, const DevPairs& pr,
                            const int32_t* numorbs, double dv, double* H, cudaStream_t st);

}  // namespace lcp
