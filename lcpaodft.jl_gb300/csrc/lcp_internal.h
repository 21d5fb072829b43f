// Internal declarations of the lcpgrid library (not part of the C ABI).
#pragma once

#include <cstdint>
#include <string>
#include <array>
#include <vector>

#include "lcpgrid.h"

namespace lcp {

// Host grid geometry: the fields of struct UCell / System_Grid
// (src/UCell.jl:1-46) plus the folded pair list the device kernels use.
struct UCell {
  int32_t nspin = 1;
  int32_t natom = 0;
  int32_t cpycell = 0;
  double lat[3][3] = {};     // rows are lattice vectors (bohr)
  double glat[3][3] = {};    // Latvecs[d,:] / Ngrid[d]
  int32_t ngrid[3] = {};
  double origin[3] = {};
  double gridvol = 0.0;
  std::vector<int32_t> atom2spe;  // 1-based species
  std::vector<double> gxyz;       // natom*3
  std::vector<double> cut;        // Atoms_Cut1
  std::vector<int32_t> numorbs;   // Total_NumOrbs

  // image cells (src/utils/Generation_ATV.jl)
  int32_t ncell = 0;
  std::vector<double> atv;       // ncell*3
  std::vector<int32_t> atv_ijk;  // ncell*3
  std::vector<int32_t> ratv;     // (2C+1)^3 -> cell

  // neighbour lists (src/UCell.jl:612-672)
  std::vector<int32_t> fnan;
  std::vector<std::vector<int32_t>> natn, ncn;  // natn 1-based

  // sphere lists (src/UCell.jl:297-411), CSR over atoms
  std::vector<int64_t> sphere_off;  // natom+1
  std::vector<int32_t> glist;       // GridListAtom (flat)
  std::vector<int32_t> clist;       // CellListAtom (flat)

  // pair list in reference order (src/UCell.jl:90-99)
  int32_t nloop = 0;
  std::vector<int32_t> pair_atom, pair_jatom, pair_cell;  // 0-based atoms
  std::vector<int64_t> block_off;                          // offset of each DM/H block
  int64_t total_hsize = 0;
  std::vector<int32_t> partner;     // pair index of (j, i, -R)
  std::vector<int64_t> numolg;      // per pair

  // folded ("unique") pairs: one of each {(i,j,R), (j,i,-R)}, with the
  // exact overlap lists of the kept orientation (CSR)
  std::vector<int32_t> uniq_pair;   // pair index kept
  std::vector<int64_t> uniq_off;    // n_unique+1
  std::vector<int32_t> uniq_g1;     // index into atom's sphere list
  std::vector<int32_t> uniq_g2;     // index into jatom's sphere list

  int32_t max_numorbs() const {
    int32_t m = 0;
    for (auto v : numorbs) m = v > m ? v : m;
    return m;
  }
  int64_t nn() const { return (int64_t)ngrid[0] * ngrid[1] * ngrid[2]; }
};

// Grid bricks for the tensor-core contractions.  The home cell is tiled by
// bricks of bdim points (at most 128; the last brick of an axis is ragged
// when bdim[d] does not divide Ngrid[d], its slots past the grid empty); the
// point slot of a brick-local coordinate l is (l0*bdim1 + l1)*bdim2 + l2.
// Each atom's sphere is covered by "blocks": the bricks of the unrolled
// lattice it touches, each holding 16 of the atom's orbitals on the brick's
// points (zero outside the sphere).  An atom with NO orbitals has
// ceil(NO/16) consecutive blocks per brick ("chunks"), each an image of its
// own ("sub-image").  A home brick sees every block whose brick maps to it,
// i.e. every chunk of every atom image touching it.  Pair tables refer to
// sub-pairs (pair, row chunk, column chunk); for atoms of <= 16 orbitals a
// sub-pair is the pair itself.
struct Bricks {
  int32_t bdim[3] = {1, 1, 1};
  int32_t nb[3] = {1, 1, 1};       // home bricks per axis
  int32_t npts = 1;                // points per brick
  int64_t nbricks = 0;
  int64_t nblocks = 0;
  int32_t max_images = 0;
  std::vector<int32_t> block_atom;   // [nblocks]
  std::vector<int32_t> point_code;   // per sphere point: block*128 + slot
  std::vector<int64_t> img_off;      // [nbricks+1]
  std::vector<int32_t> img_block;    // block of each image of a home brick (blocks are numbered in image order)
  std::vector<int32_t> img_atom;
  std::vector<int64_t> tab_off;      // [nbricks+1] offsets of the m x m pair tables
  std::vector<int32_t> tab_pair;     // sub-pair of sub-images (s, t), -1 if none
  // grid-H partial blocks: one per (brick, s <= t) image pair that is a pair
  std::vector<int32_t> tab_slot;     // m x m per brick: slot within the brick, -1 if none
  std::vector<int64_t> slot_base;    // [nbricks+1]
  // sub-pairs of the neighbour pairs
  int64_t nsub = 0;
  std::vector<int64_t> sub_off;      // [nloop+1]: first sub-pair of each pair
  std::vector<int32_t> sub_pair;     // [nsub] pair of each sub-pair
  std::vector<int32_t> sub_chunks;   // [nsub] (row chunk << 8) | column chunk
  // 16 x 16 sub-blocks of the folded pairs' H blocks (kept orientation)
  std::vector<int64_t> sb_off;       // [n_unique+1]
  std::vector<int32_t> sb_fold;      // [nsb] folded pair of each sub-block (reduction order: longest first)
  std::vector<int32_t> sb_chunks;    // [nsb] (row chunk << 8) | column chunk
  std::vector<int64_t> red_off;      // [nsb+1] CSR of slots per sub-block
  std::vector<int64_t> red_slot;     // global slot * 2 + (1 if the slot enters transposed)
};
// Bricks of the given shape (ragged at the upper edge of an axis whose
// Ngrid the side does not divide); shape == nullptr or shape[0] <= 0: the
// predicted best shape with at most kMaxBrickImages sub-images per brick
// (the kernels take any count; the bound keeps a brick's m x m pair tables
// small).
constexpr int kMaxBrickImages = 512;
std::string build_bricks(const UCell& u, Bricks& b, const int32_t* shape = nullptr);
// Brick shapes (sides <= 8, 16..128 points) ranked by predicted cost.
double brick_shape_cost(const UCell& u, const int32_t* bd);
std::vector<std::array<int32_t, 3>> brick_shape_candidates(const UCell& u, std::vector<double>* costs);

// Builds everything above; returns an error message or "".
std::string build_ucell(UCell& u, int32_t nspin, const double* latvecs, int32_t natom,
                        const int32_t* atom2spe, const double* gxyz, const double* cut,
                        const int32_t* ngrid, const double* origin, const int32_t* numorbs);

// Overlap lists of one pair in reference orientation and order
// (GListTAtoms1/2 of src/UCell.jl:425-516).
void pair_overlap(const UCell& u, int32_t pair, std::vector<int32_t>& g1, std::vector<int32_t>& g2);

void set_error(const std::string& msg);

// The parts of UCell(...): build_ucell = build_ucell_head (checks, image
// cells, neighbour and pair lists), then the sphere lists (Calc_AtomsGrid)
// and the overlap lists (Calc_AtomOverlap_Grid), on the host or the device.
std::string build_ucell_head(UCell& u, int32_t nspin, const double* latvecs, int32_t natom,
                             const int32_t* atom2spe, const double* gxyz, const double* cut,
                             const int32_t* ngrid, const double* origin, const int32_t* numorbs);
void build_spheres_host(UCell& u);
void build_overlaps_host(UCell& u);
// The grid-index box [nmin, nmax] Calc_AtomsGrid scans for atom a.
void atom_box(const UCell& u, int a, int nmin[3], int nmax[3]);

// Calc_Diff_Coef (src/XC/GGA_PBE.jl:1-39): the x, y, z first-derivative
// weights [3][27] of the tri-quadratic fit through the 27 neighbours of a grid
// point, for grid vectors gtv (rows).  False if the fit matrix is singular.
bool calc_diff_coef(const double gtv[3][3], double out[81]);

}  // namespace lcp
