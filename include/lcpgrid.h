/*
 * lcpgrid.h -- C ABI of the GB300 (sm_103a) real-space grid path of LCPAODFT.jl.
 *
 * Plain C types only: pointers, sizes, int32/int64/double.  Every call
 * returns an lcp_status; no exception crosses the ABI.  lcp_last_error()
 * gives the message of the last failing call on the calling thread.
 *
 * Conventions shared with the reference (LCPAODFT.jl):
 *   - grids are C-order flat vectors of length NN = N1*N2*N3, index
 *     n1*N2*N3 + n2*N3 + n3 (src/UCell.jl:380);
 *   - atoms are 1-based where the reference stores them 1-based (atom2spe,
 *     natn); grid/cell/overlap indices are 0-based as the reference stores
 *     them (GridListAtom, CellListAtom, GListTAtoms1/2);
 *   - DM and H use the flat pair-block layout of the reference: pairs in
 *     (atom 1..Natom, neighbour 1..FNAN+1) order, each block NO(jatom) rows x
 *     NO(atom) columns, column-major (src/Hamiltonian.jl:16-38,
 *     src/Matrix/Set_Density_Grid.jl:94-97);
 *   - SpinPol "off"/"on"/"nc" is LCP_SPIN_OFF/ON/NC with 1/2/4 channels.
 *
 * Threading: one lcp_ctx per host thread; calls on one context run in order
 * on its CUDA stream.  Host buffers passed to a call are read or written
 * before the call returns and are not retained.
 */
#ifndef LCPGRID_H
#define LCPGRID_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t lcp_status;
enum {
  LCP_OK = 0,
  LCP_EINVAL = 1,    /* invalid argument (the reference raises error()) */
  LCP_ENOMEM = 2,    /* host or device allocation failed */
  LCP_EDEVICE = 3,   /* CUDA error */
  LCP_ETIMEDOUT = 4, /* a bounded device wait gave up */
  LCP_ENOTSUP = 5,   /* unsupported shape or mode */
  LCP_ESTATE = 6     /* object used in the wrong state */
};

enum { LCP_SPIN_OFF = 0, LCP_SPIN_ON = 1, LCP_SPIN_NC = 2 };
enum { LCP_XC_LDA = 0, LCP_XC_LSDA = 1, LCP_XC_GGA_PBE = 2 };
/* arithmetic of the pair contractions (density assembly, grid H) */
enum { LCP_PREC_FP64 = 0, LCP_PREC_FP32 = 1, LCP_PREC_BF16X3 = 2 };

typedef struct lcp_ucell lcp_ucell; /* host grid geometry (struct UCell) */
typedef struct lcp_ctx lcp_ctx;     /* device context: stream, handles, workspaces */
typedef struct lcp_orbs lcp_orbs;   /* device orbital tables (PackedOrbitalsGrid) */
typedef struct lcp_job lcp_job;     /* device-resident SCF grid-step state */

/* Radial tables of one species: the fields of struct PAO the grid path reads
 * (src/Atoms/Read_PAO.jl:1-18). */
typedef struct {
  int32_t max_l;         /* Spe_MaxL_Basis, 0..3 */
  int32_t num_basis[4];  /* Spe_Num_Basis[l] */
  int32_t num_mesh;      /* Spe_Num_Mesh_PAO (>= 8) */
  const double* rv;      /* Spe_PAO_RV[num_mesh], increasing */
  const double* rwf;     /* Spe_PAO_RWF: for l, for p < num_basis[l]: num_mesh values */
} lcp_pao;

const char* lcp_last_error(void);
const char* lcp_version(void);

/* ---------------------------------------------------------------- geometry */

/* UCell(Nspin, Latvecs, Natom, atom2spe, Gxyz, Atoms_Cut1, Ngrid, Grid_Origin;
 *       Total_NumOrbs)  -- src/UCell.jl:210-294 (one MPI rank).
 * latvecs: 3x3 row vectors (row-major); gxyz: natom x 3 (bohr);
 * atom2spe: 1-based species per atom; total_numorbs may be NULL (zeros). */
lcp_status lcp_ucell_create(int32_t nspin, const double* latvecs, int32_t natom,
                            const int32_t* atom2spe, const double* gxyz,
                            const double* atoms_cut1, const int32_t* ngrid,
                            const double* grid_origin, const int32_t* total_numorbs,
                            lcp_ucell** out);
void lcp_ucell_destroy(lcp_ucell* ucell);

typedef struct {
  int32_t cpycell;      /* System_Grid.CpyCell */
  int32_t natom;
  int32_t nloop;        /* number of (atom, neighbour) pairs, System_Grid.Nloop */
  int32_t ncell;        /* (2*CpyCell+1)^3 */
  int32_t ngrid[3];
  int32_t max_numorbs;
  int64_t total_hsize;  /* System_Grid.Total_Hsize */
  int64_t sum_gridn;    /* sum of GridN_Atom */
  int64_t sum_numolg;   /* sum of MPI_NumOLG over all pairs */
  int64_t n_unique;     /* pairs kept after folding (i,j,R) with (j,i,-R) */
  double gridvol;       /* System_Grid.GridVol */
} lcp_ucell_info;
lcp_status lcp_ucell_get_info(const lcp_ucell* ucell, lcp_ucell_info* info);

/* Integer fields of UCell, copied to dst[count]; `index` selects the atom or
 * pair for per-atom / per-pair lists (0-based), ignored otherwise. */
enum {
  LCP_F_FNAN = 0,         /* [natom] */
  LCP_F_NATN = 1,         /* per atom [FNAN+1], 1-based atoms */
  LCP_F_NCN = 2,          /* per atom [FNAN+1] */
  LCP_F_GRIDN_ATOM = 3,   /* [natom] */
  LCP_F_GRIDLIST = 4,     /* per atom [GridN] */
  LCP_F_CELLLIST = 5,     /* per atom [GridN] */
  LCP_F_PAIR_ATOM = 6,    /* [nloop], 1-based */
  LCP_F_PAIR_NATN = 7,    /* [nloop], 1-based */
  LCP_F_PAIR_NCN = 8,     /* [nloop] */
  LCP_F_NUMOLG = 9,       /* [nloop] */
  LCP_F_GLIST1 = 10,      /* per pair [NumOLG] (GListTAtoms1) */
  LCP_F_GLIST2 = 11,      /* per pair [NumOLG] (GListTAtoms2) */
  LCP_F_ATV_IJK = 12      /* [ncell*3] */
};
lcp_status lcp_ucell_get_int(const lcp_ucell* ucell, int32_t field, int64_t index,
                             int32_t* dst, int64_t count);
lcp_status lcp_ucell_get_atv(const lcp_ucell* ucell, double* dst /* [ncell*3] */);
/* Grid-brick tiling of the tensor-core path: info[14] = brick dims (3), bricks
 * per axis (3), points per brick, bricks, table blocks, max atom images of a
 * brick, total images, image pairs that are neighbour pairs, partial H blocks
 * (FP32 scratch slots of 1 KB), split-D sub-pairs. */
lcp_status lcp_ucell_get_bricks(const lcp_ucell* ucell, int64_t* info);
/* Brick shapes (sides <= 8, 16..128 points; the last brick of an axis is
 * ragged where the side does not divide Ngrid) ranked by the predicted cost
 * of the tensor-core passes: up to `max` shapes (3 ints each) and their costs
 * (arbitrary units; may be NULL). */
lcp_status lcp_brick_shape_candidates(const lcp_ucell* ucell, int32_t max, int32_t* shapes, double* cost,
                                      int32_t* n);

/* UCell(...) with Calc_AtomsGrid and Calc_AtomOverlap_Grid (src/UCell.jl:297-516)
 * run on the context's GPU: the same object as lcp_ucell_create, with the
 * same lists bit for bit.  LCP_ENOTSUP when an atom's grid box reaches image
 * cells outside -CpyCell..CpyCell-1 (where the reference's Find_CGrids!
 * leaves its table or takes its out-of-range branch); lcp_ucell_create
 * handles those cells. */
lcp_status lcp_ucell_create_device(lcp_ctx* ctx, int32_t nspin, const double* latvecs, int32_t natom,
                                   const int32_t* atom2spe, const double* gxyz, const double* atoms_cut1,
                                   const int32_t* ngrid, const double* grid_origin, const int32_t* total_numorbs,
                                   lcp_ucell** out);

/* Calc_Ngrid(Ecut, Latvecs) -- src/utils/Calc_Ngrid.jl:1-76 */
lcp_status lcp_calc_ngrid(double ecut, const double* latvecs, int32_t* ngrid_out);

/* ---------------------------------------------------------------- context */

lcp_status lcp_ctx_create(int32_t device, lcp_ctx** out);
void lcp_ctx_destroy(lcp_ctx* ctx);
/* Run subsequent work on an external cudaStream_t (NULL: the context's own). */
lcp_status lcp_ctx_set_stream(lcp_ctx* ctx, void* stream);
lcp_status lcp_ctx_set_precision(lcp_ctx* ctx, int32_t precision);
lcp_status lcp_ctx_synchronize(lcp_ctx* ctx);
/* Number of kernels this library launched on the context so far. */
int64_t lcp_ctx_launch_count(const lcp_ctx* ctx);

/* ---------------------------------------------------------------- the grid path */

/* Set_Orbitals_Grid(pao, ucell) and, with with_grad != 0, Set_dOrbitals_Grid
 * (src/Matrix/Set_Orbitals_Grid.jl:26-277, src/Matrix/Set_dOrbitals_Grid.jl:1-362).
 * paos[spe-1] is the species of atom2spe. Tables stay on the device. */
lcp_status lcp_set_orbitals_grid(lcp_ctx* ctx, const lcp_ucell* ucell, int32_t nspecies,
                                 const lcp_pao* paos, int32_t with_grad, lcp_orbs** out);
void lcp_orbs_destroy(lcp_orbs* orbs);
/* Copy one atom's table to the host, point-major [GridN x NO] (the memory of
 * PackedOrbitalsGrid.data[atom]).  component: 0 = phi, 1..3 = d/dx, d/dy, d/dz. */
lcp_status lcp_orbs_download(lcp_ctx* ctx, const lcp_orbs* orbs, int32_t component,
                             int32_t atom, double* dst, int64_t count);

/* A radial table on a log mesh, as KumoF reads it (src/utils/KumoF.jl). */
typedef struct {
  int32_t num_mesh;  /* mesh points (>= 8) */
  const double* xv;  /* log radii (Spe_PAO_XV / Spe_VPS_XV) */
  const double* rv;  /* radii (Spe_PAO_RV / Spe_VPS_RV) */
  const double* yv;  /* values in the (num_mesh + 4)-long layout (Spe_Atomic_Den / Spe_Atomic_PCC) */
} lcp_radial;

/* Set_AdenPCC_Grid(SpinPol, Init_Atoms_Nspin, Init_Atoms_Angle, pao, pspot, ucell)
 * (src/Matrix/Set_AdenPCC_Grid.jl:1-142) on the device: the atomic density,
 * the partial-core density and the initial Density_Grid (1, 2 or 4 channels).
 * init_atoms_nspin[atom*2 + {0,1}] = (Nu, Nd); init_atoms_angle[atom*2 + {0,1}]
 * = (theta, phi), read for "nc" only (may be NULL otherwise).  atomic_den[spe]
 * and atomic_pcc[spe] are the species' tables (atom2spe, 1-based).  Outputs
 * are host arrays of NN doubles; every point sums its atoms' terms in the
 * reference's order. */
lcp_status lcp_set_adenpcc_grid(lcp_ctx* ctx, const lcp_ucell* ucell, int32_t spinpol,
                                const double* init_atoms_nspin, const double* init_atoms_angle, int32_t nspecies,
                                const lcp_radial* atomic_den, const lcp_radial* atomic_pcc, double* adensity_grid,
                                double* pccdensity_grid, double* const* density_grid);

/* Set_Density_Grid!(SpinPol, ucell, Orbs_Grid, DM, Density_Grid)
 * (src/Matrix/Set_Density_Grid.jl:1-304).  dm[s]: Total_Hsize doubles;
 * density_grid[s]: NN doubles, overwritten. */
lcp_status lcp_set_density_grid(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs,
                                int32_t spinpol, const double* const* dm,
                                double* const* density_grid);

/* Solve_Poisson!(SpinPol, dft_mixing, Density_Grid, ADensity_Grid, dVHart_Grid)
 * (src/Poisson.jl:1-26).  recvecs = 2*pi*inv(Latvecs') row vectors. */
lcp_status lcp_solve_poisson(lcp_ctx* ctx, const int32_t* ngrid, const double* recvecs,
                             int32_t spinpol, const double* const* density_grid,
                             const double* adensity_grid, double* dvhart_grid);
/* Inner Solve_Poisson!(Ngrid, Recvecs, Density_xyz, dVHart_Grid) for a real
 * Density_xyz (src/Poisson.jl:29-108). */
lcp_status lcp_solve_poisson_xyz(lcp_ctx* ctx, const int32_t* ngrid, const double* recvecs,
                                 const double* density_xyz, double* dvhart_grid);

/* Set_XC_Grid!(xc_func::XC_LDA|XC_LSDA, PCCDensity_Grid, Density_Grid)
 * (src/XC/XC_Func.jl:111-145). nc additionally reads Density_Grid[3:4]. */
lcp_status lcp_set_xc_grid(lcp_ctx* ctx, int32_t xc, int32_t spinpol, int64_t nn,
                           const double* pcc, const double* const* density_grid,
                           double* const* vxc_grid);

/* diagonalize_nc_density!(Density_Grid) (src/Matrix/Set_Density_Grid.jl:243-261):
 * the four "nc" channels (Re11, Re22, Re12, Im12), host arrays of nn doubles,
 * become (Nup, Ndown, theta, phi) in place (EulerAngle_Spin,
 * src/utils/EulerAngle_Spin.jl:1-6). */
lcp_status lcp_diagonalize_nc_density(lcp_ctx* ctx, int64_t nn, double* const* density_grid);

/* Calc_Diff_Coef(gLatvecs) (src/XC/GGA_PBE.jl:1-39), the Diff_Coef of
 * XC_Func("GGA_PBE", ...) (src/XC/XC_Func.jl:87-104): diff_coef[3*27] = the
 * x, y, z gradient weights of the 27-point stencil for the grid vectors
 * glatvecs (3x3 row-major, row i = Latvecs row i / Ngrid[i]).  Host only. */
lcp_status lcp_calc_diff_coef(const double* glatvecs, double* diff_coef);

/* Set_XC_Grid!(xc_func::XC_GGA_PBE, PCCDensity_Grid, Density_Grid)
 * (src/XC/XC_Func.jl:148-160): Set_dDensity_Grid! then Set_Vxc_GGA_PBE!
 * (src/XC/GGA_PBE.jl:53-193, 274-462) on the Ngrid grid.  vxc_grid: 1 ("off"),
 * 2 ("on") or 4 ("nc", which also reads Density_Grid[3:4]) channels.
 * ddensity_grid and dexc_dgd (each NULL, or 3 pointers per spin, [spin][xyz],
 * one spin for "off", two otherwise) receive xc_func.dDensity_Grid and
 * xc_func.dEXC_dGD.  pcc may be NULL (zero). */
lcp_status lcp_set_xc_grid_gga(lcp_ctx* ctx, int32_t spinpol, const int32_t* ngrid, const double* diff_coef,
                               const double* pcc, const double* const* density_grid, double* const* vxc_grid,
                               double* const* ddensity_grid, double* const* dexc_dgd);

/* Set_Vpot_Grid!(xc_func, dVHart_Grid, Vpot_Grid) (src/Matrix/Set_Vpot_Grid.jl:1-19);
 * vna (may be NULL) is added to the spin-diagonal channels. */
lcp_status lcp_set_vpot_grid(lcp_ctx* ctx, int32_t spinpol, int64_t nn, const double* dvhart,
                             const double* const* vxc, const double* vna, double* const* vpot);

/* Calc_MatrixElements_dVH_Vxc_{off,on,nc}!(ucell, Orbs_Grid, Vpot_Grid, MPI_Hks)
 * (src/Hamiltonian.jl:235-429): hks[ch] (Total_Hsize) overwritten with the grid
 * part, scaled by GridVol. */
lcp_status lcp_calc_matrix_elements(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs,
                                    int32_t spinpol, const double* const* vpot, double* const* hks);

/* Force3_nospin / Force3_spin / Force3_nc (src/Force.jl:405-566 with
 * _Calc_Force3_Blocked_Kernel!, src/Force.jl:3344-3394): the grid force term
 * force[atom*3 + xyz] (Natom x 3, row-major), in FP64 whatever the context's
 * precision.  vpot[c] (NN doubles) are the channels' potentials as the
 * reference passes them -- off: Vpot; on: Vpot up, down; nc: dVHart + Vxc1,
 * dVHart + Vxc2, Vxc3, Vxc4 -- and dm[c] the flat pair-block density
 * matrices.  The orbitals must carry gradient tables (tabulated with
 * grad = 1, Set_dOrbitals_Grid), else LCP_ESTATE.  Like the reference, the
 * term is the energy's gradient (f_s d<D,H>/dR with V fixed). */
lcp_status lcp_calc_force3(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs, int32_t spinpol,
                           const double* const* vpot, const double* const* dm, double* force);

/* Calc_EH1 (src/Energy.jl:655-666) and Calc_EXC1 (src/Energy.jl:669-700). */
lcp_status lcp_calc_eh1(lcp_ctx* ctx, int32_t spinpol, int64_t nn, double gridvol,
                        const double* adensity, const double* const* density,
                        const double* dvhart, double* eh1);
lcp_status lcp_calc_exc1(lcp_ctx* ctx, int32_t xc, int32_t spinpol, int64_t nn, double gridvol,
                         const double* adensity, const double* pcc,
                         const double* const* density, double* exc /* [2] */);
/* Calc_EXC1(SpinPol, xc_type, system_grid, ...) (src/Energy.jl:669-700) with the
 * system grid given as Ngrid and Latvecs (3x3 row-major; GridVol = |det| / NN):
 * every xc type, GGA_PBE included (its energy per particle needs the gradient
 * stencil, src/XC/XC_Func.jl:193-215). */
lcp_status lcp_calc_exc1_grid(lcp_ctx* ctx, int32_t xc, int32_t spinpol, const int32_t* ngrid,
                              const double* latvecs, double gridvol, const double* adensity, const double* pcc,
                              const double* const* density, double* exc /* [2] */);

/* ---------------------------------------------------------------- device-resident step */

/* One SCF grid step with all state on the device: density from D, Poisson,
 * xc, potential (+ optional V_na), grid H and the FP64 energy terms.  The
 * inputs adensity/pcc/vna (NN doubles each, may be NULL = zero) are copied at
 * creation.  xc: LDA ("off"), LSDA ("on", "nc") or GGA_PBE (any; its
 * gradient stencil comes from the cell's Latvecs and Ngrid).  "nc" carries
 * four DM/density/potential/H channels: the density is diagonalized
 * (diagonalize_nc_density!) before Poisson and xc, as src/KSsolve_SCF.jl:252-255
 * does, and the xc potentials are rotated into the four channels. */
lcp_status lcp_job_create(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs,
                          int32_t spinpol, int32_t xc, const double* adensity,
                          const double* pcc, const double* vna, lcp_job** out);
void lcp_job_destroy(lcp_job* job);
/* Host -> device copy of the density matrices (Nspin x Total_Hsize). */
lcp_status lcp_job_set_dm(lcp_ctx* ctx, lcp_job* job, const double* const* dm);
/* Launch one grid step on the context stream (asynchronous).  Any context of
 * the job's device may run it (its workspaces and FFT plans are used); steps
 * of one job must not overlap.  From a job's second step on a context the
 * launches are replayed as one CUDA graph (lcp_ctx_set_step_graphs). */
lcp_status lcp_job_step(lcp_ctx* ctx, lcp_job* job);
/* The same step with CUDA events between its stages (synchronises); stage_ms[6] =
 * density, Poisson, xc+potential (with the energy partial sums of the same
 * pass), energy sums (their final reduction), grid H, <D,H> + job energy
 * (the stage names of the reference's TimerOutputs sections). */
lcp_status lcp_job_step_timed(lcp_ctx* ctx, lcp_job* job, double* stage_ms);
/* One split-BF16 step with CUDA events around its tensor-core kernels alone
 * (synchronises): ms[0] = the density kernel's time summed over the spin
 * channels, ms[1] = the grid-H kernel's, without the D symmetrisation, the V
 * weights and the partial-block reduction around them.  LCP_ENOTSUP unless
 * the context runs split-BF16.  Replaces nothing of the reference (a
 * measurement of this library's kernels). */
lcp_status lcp_job_tc_kernel_ms(lcp_ctx* ctx, lcp_job* job, double* ms);
/* Energies of the last step: [E_H1, EXC1[1], EXC1[2], sum_s <D_s,H_s>, E_grid]. */
lcp_status lcp_job_energies(lcp_ctx* ctx, lcp_job* job, double* out5);
/* The energies without waiting: an asynchronous copy on the context's stream
 * (out5 should be pinned host memory; valid once the stream reaches it). */
lcp_status lcp_job_energies_async(lcp_ctx* ctx, lcp_job* job, double* out5);
/* Builds what the context's precision needs of the job's orbital tables
 * (split-BF16 brick tables, FP32 copy) ahead of the first step. */
lcp_status lcp_job_prepare(lcp_ctx* ctx, lcp_job* job);
/* Device bytes held by the job and its orbital tables (admission by HBM
 * footprint). */
lcp_status lcp_job_footprint(const lcp_job* job, int64_t* bytes);
/* Waits for the context's stream and reports (and clears) a device-side error
 * of its kernels (a bounded wait that gave up: LCP_ETIMEDOUT). */
lcp_status lcp_ctx_check_status(lcp_ctx* ctx);
/* Device -> host copies of the last step's outputs. */
lcp_status lcp_job_get_density(lcp_ctx* ctx, lcp_job* job, double* const* density);
lcp_status lcp_job_get_hks(lcp_ctx* ctx, lcp_job* job, double* const* hks);
lcp_status lcp_job_get_vpot(lcp_ctx* ctx, lcp_job* job, double* const* vpot);

/* Measured FP64 FMA throughput of the device (TFLOP/s), a roofline denominator
 * for the FP64 contractions. */
lcp_status lcp_probe_fp64_tflops(lcp_ctx* ctx, double* tflops);
/* Tensor-core self-test: d[128 x n] = bf16(a[128 x k]) * bf16(b[n x k])^T with the
 * operands staged K-major or MN-major, core matrices ordered K-groups outer
 * (order 0) or MN-groups outer (order 1); row-major host inputs, FP32 result. */
lcp_status lcp_tc_selftest(lcp_ctx* ctx, int32_t a_mn_major, int32_t b_mn_major, int32_t order, int32_t n,
                           int32_t k, const float* a, const float* b, float* d);
/* The xc functional per point, as the grid step's xc pass evaluates it: LDA
 * (xc = LCP_XC_LDA, density 2 (up + pcc)) or LSDA (up + pcc, dn + pcc), in
 * FP64 (double_float = 0: the FP64 drop-in) or in double-float (1: the
 * precision forms).  out[3 i] = exc, out[3 i + 1] = vxc up, out[3 i + 2] =
 * vxc down (0 for LDA); host arrays of n points; dn ignored for LDA, pcc may
 * be NULL.  Replaces nothing of the reference: it checks one arithmetic
 * against the other (src/XC/LDA_CA.jl:4-41, src/XC/LSDA_CA.jl:1-138). */
lcp_status lcp_xc_selftest(lcp_ctx* ctx, int32_t xc, int32_t double_float, int64_t n, const double* up,
                           const double* dn, const double* pcc, double* out);

/* ---------------------------------------------------------------- serving */

/* Serving engine for SCF grid-step requests on many device-resident
 * structures (the serving form; the reference has no serving layer).
 * `nslots` execution slots, each a context of its own (stream and
 * workspaces) at `precision` with a worker thread, take pending requests in
 * arrival order as they and their structures free up; at LCP_PREC_BF16X3 a
 * slot runs the requests it takes (up to lcp_server_set_max_batch) as one
 * batched grid step, and the slots' steps overlap on the device.  Structures
 * are admitted by device footprint against `budget_bytes`. */
typedef struct lcp_server lcp_server;
lcp_status lcp_server_create(int32_t device, int32_t nslots, int32_t precision, int64_t budget_bytes,
                             lcp_server** out);
/* Waits for the requests in flight, then frees the server (not the jobs). */
void lcp_server_destroy(lcp_server* srv);
/* Adds a job (a structure with its orbital tables and step buffers, created
 * by the caller, who keeps ownership): admitted now if its footprint (with
 * the precision's tables) fits the free budget, else queued for admission
 * with its requests until removals free the budget (lcp_server_state);
 * LCP_ENOMEM only when it exceeds the whole budget.  nspin / hsize: channels
 * and Total_Hsize of its D. */
lcp_status lcp_server_add(lcp_server* srv, lcp_job* job, int32_t nspin, int64_t hsize, int32_t* id);
/* Releases a structure's budget (LCP_ESTATE while it has requests queued)
 * and admits queued structures that now fit, in order. */
lcp_status lcp_server_remove(lcp_server* srv, int32_t id);
/* Queues one grid step of structure `id` with density matrices dm[nspin]
 * (copied; the caller's buffers are free on return). */
lcp_status lcp_server_submit(lcp_server* srv, int32_t id, const double* const* dm, uint64_t tag);
/* Completed requests (up to max; waits up to wait_ms for the first): tags,
 * energies[5 each] (as lcp_job_energies) and submission-to-result latency. */
lcp_status lcp_server_poll(lcp_server* srv, int32_t max, int32_t wait_ms, uint64_t* tags, double* energies,
                           double* latency_ms, int32_t* n);
/* out4 = submitted, completed, resident bytes, budget. */
lcp_status lcp_server_stats(lcp_server* srv, int64_t* out4);
/* The serving form's own controls; no counterpart in the reference.
 * lcp_server_state: 0 admitted, 1 waiting in the admission queue (the
 * structure did not fit the free budget when added; removals admit queued
 * structures in order), 2 being admitted. */
lcp_status lcp_server_state(lcp_server* srv, int32_t id, int32_t* state);
/* Requests per batched step: each slot takes up to max_batch pending requests
 * of idle admitted structures with one SpinPol and xc and runs them as one
 * batched grid step (split-BF16 servers only; default 16 at LCP_PREC_BF16X3,
 * 1 otherwise: LCP_ENOTSUP for more than 1 at another precision). */
lcp_status lcp_server_set_max_batch(lcp_server* srv, int32_t max_batch);
/* out5 = batched steps run (more than one request), requests they carried,
 * structures waiting for admission, host microseconds spent assembling those
 * batches and their total wall microseconds (assembly to completion). */
lcp_status lcp_server_batch_stats(lcp_server* srv, int64_t* out5);

/* ---------------------------------------------------------------- brick tiling of the split-BF16 path */

/* Sets the brick shape of the orbitals' split-BF16 tables (shape NULL or
 * {0,0,0}: the predicted best); the tables are rebuilt on next use. */
lcp_status lcp_orbs_set_brick_shape(lcp_ctx* ctx, lcp_orbs* orbs, const int32_t* shape);
/* The brick shape in use (builds the tables if needed). */
lcp_status lcp_orbs_get_brick_shape(lcp_ctx* ctx, lcp_orbs* orbs, int32_t* shape);
/* Autotuner: times the density and matrix-element passes on the device for
 * the `ncand` best predicted shapes (skipping shapes whose bricks see more
 * atom images than the kernels hold) and keeps the fastest; shape_out[3] and
 * ms_out (its time for one density + one H pass) may be NULL. */
lcp_status lcp_orbs_autotune_bricks(lcp_ctx* ctx, lcp_orbs* orbs, int32_t ncand, int32_t* shape_out,
                                    double* ms_out);
/* Builds the split-BF16 tables, then frees the FP64 (and FP32, gradient)
 * orbital tables: the orbitals then serve the split-BF16 path only (other
 * precisions, downloads and shape changes return LCP_ESTATE). */
lcp_status lcp_orbs_release_fp64(lcp_ctx* ctx, lcp_orbs* orbs);

/* ---------------------------------------------------------------- batching */

/* Batched grid step over the device-resident jobs of many cells (the
 * batching form; the reference steps one cell at a time).  Each
 * stage runs once for all cells: one persistent tensor-core launch over the
 * bricks of every cell for the density and for the matrix elements, one
 * FFT Poisson solve per grid shape, tiled grid kernels and FP64 reductions
 * over all cells.  The step is captured once as a CUDA graph and replayed.  Results
 * land in the jobs' own buffers (read them with lcp_job_get_* /
 * lcp_job_energies); each cell's density, H and energy sums are computed as
 * in a single-cell split-BF16 step.  The jobs (same SpinPol and xc, split-BF16
 * context) stay owned by the caller and must outlive the batch; their D is
 * set with lcp_job_set_dm. */
typedef struct lcp_batch lcp_batch;
enum { LCP_BATCH_GRAPH = 0, LCP_BATCH_EAGER = 1 };
/* scratch_bytes: budget for the FP32 partial H blocks (1 KB each) that the
 * matrix-element pass keeps until their reduction; the cells are taken in
 * waves that fit it, one launch per wave (0: no limit, one wave). */
lcp_status lcp_batch_create(lcp_ctx* ctx, int32_t njobs, lcp_job* const* jobs, int64_t scratch_bytes,
                            lcp_batch** out);
void lcp_batch_destroy(lcp_batch* batch);
/* One step of every cell on the context's stream (asynchronous).
 * LCP_BATCH_GRAPH: replay the captured graph (the first call runs eagerly and
 * captures); LCP_BATCH_EAGER: launch the kernels one by one. */
lcp_status lcp_batch_step(lcp_ctx* ctx, lcp_batch* batch, int32_t mode);
/* One eager step with CUDA events between its stages (synchronises):
 * stage_ms[6] as lcp_job_step_timed, for all cells together. */
lcp_status lcp_batch_step_timed(lcp_ctx* ctx, lcp_batch* batch, double* stage_ms);
/* Waits for the stream; reports (and clears) a device-side timeout. */
lcp_status lcp_batch_check_status(lcp_ctx* ctx, lcp_batch* batch);
/* energies[5 * njobs]: each job's lcp_job_energies, in the batch's order. */
lcp_status lcp_batch_energies(lcp_ctx* ctx, lcp_batch* batch, double* energies);
/* out8 = cells, grid-shape groups, bricks, own kernels per step, workspace
 * bytes, graph captured (0/1), H sub-blocks, waves of the H pass. */
lcp_status lcp_batch_info(const lcp_batch* batch, int64_t* out8);

/* Split-BF16 density that allocates no device memory.  No counterpart in the
 * reference: it is for callers that cannot call cudaMalloc at call time --
 * hosts whose own pool allocator owns the device memory, and serving loops
 * that cannot afford the device-wide synchronisation cudaMalloc/cudaFree may
 * cause.  Same result as lcp_set_density_grid at LCP_PREC_BF16X3 (whatever
 * the context's precision), but dm_dev[s] (Total_Hsize doubles) and
 * density_grid_dev[s] (NN doubles, overwritten) are DEVICE pointers owned by
 * the caller.  Scratch lives in one fixed 16 MiB device array per device,
 * held from the library's load on that device until exit; it fits cells of
 * up to 10921 neighbour pairs (Nloop) and larger ones are rejected with
 * LCP_EINVAL.  The orbitals' split-BF16 tables must already exist (any
 * allocating split-BF16 call on them builds them), else LCP_ESTATE.
 * The call is synchronous: it copies the error word to the host and waits for
 * the context's stream before it returns, so it cannot be captured into a
 * CUDA graph.  The first call on a context looks up the array's device
 * address (cudaGetSymbolAddress); while another thread captures a stream in
 * the global capture mode, that first call must not run.  Every call on a
 * device shares the array and leaves its contents behind: calls that overlap
 * on the GPU (other host threads, other contexts of that device) race and
 * must be serialised by the caller.  Calls after cudaDeviceReset need a
 * context created after the reset. */
lcp_status lcp_set_density_grid_noalloc(lcp_ctx* ctx, const lcp_ucell* ucell, const lcp_orbs* orbs,
                                        int32_t spinpol, const double* const* dm_dev,
                                        double* const* density_grid_dev);

/* Device times (ms, CUDA events) of the orbitals' last tabulation kernel and
 * of their split-BF16 table build (0 until built).  No counterpart in the
 * reference (its TimerOutputs timers time the whole functions). */
lcp_status lcp_orbs_timings(const lcp_orbs* orbs, double* out2);

/* For tests of the failure path only; no counterpart in the reference.
 * poll_limit (0: the default of 2^24 polls) bounds every wait of the
 * split-BF16 density kernel on this context; stall = 1 makes one of its
 * epilogue warps withhold its stage releases, so the producers' waits run out
 * and the kernel unwinds: it records LCP_ETIMEDOUT in the context's error
 * word, stops every role, waits (bounded) for its copies and MMAs in flight,
 * frees its tensor memory and returns, and the call returns LCP_ETIMEDOUT.
 * Off (0, 0) by default; set it back to (0, 0) to run normally. */
lcp_status lcp_ctx_set_fault_test(lcp_ctx* ctx, uint32_t poll_limit, int32_t stall);

/* The arithmetic of this context's drop-in GGA-PBE entry points
 * (lcp_set_xc_grid_gga, lcp_calc_exc1_gga): 0 = FP64, the reference's (the
 * default); 1 = double-float on the FP32 pipe with FP64 sums, as the
 * precision forms' grid step evaluates GGA-PBE (about 2^-44 relative to
 * FP64).  The grid step follows its precision form
 * whatever this says.  Replaces nothing of the reference (an option of this
 * library, src/XC/XC_PBE.jl:187-476, src/XC/GGA_PBE.jl:53-462). */
lcp_status lcp_ctx_set_xc_arithmetic(lcp_ctx* ctx, int32_t double_float);

/* Whether lcp_job_step replays its launches as a CUDA graph (1, the default)
 * or launches them one by one (0).  Either gives the same results; the graph
 * is captured at a job's second step on a context and captured again when
 * the context's stream or options, or any device buffer of the library,
 * changed.  Replaces nothing of the reference (an option of this library). */
lcp_status lcp_ctx_set_step_graphs(lcp_ctx* ctx, int32_t on);

/* The check build (liblcpgrid_check.so, compiled with LCP_BOUNDS_CHECK) tests
 * every index the pair and tensor-core kernels gather with (lens entries,
 * sphere-list grid indices, DM/H block offsets, split-D pair indices, table
 * blocks, partial-block slots, grid writes) and records the first violation
 * instead of making the access: word = (site << 56) | (index + 1), 0 when
 * none; read and cleared here after the context's stream completes.
 * LCP_ENOTSUP in the normal build.  No counterpart in the reference. */
lcp_status lcp_bounds_check_status(lcp_ctx* ctx, int64_t* word);

/* Device allocations (cudaMalloc calls) the library has made since it was
 * loaded, over all contexts: a diagnostic for callers that must see none in
 * a call (lcp_set_density_grid_noalloc).  No counterpart in the reference. */
lcp_status lcp_device_alloc_count(int64_t* count);

#ifdef __cplusplus
}
#endif

#endif /* LCPGRID_H */
