// Host-side grid geometry: image cells, neighbour lists, cutoff-sphere point
// lists and pair overlap lists.  This is the UCell construction of
// LCPAODFT.jl (src/UCell.jl:210-294) for one process, computed once per
// geometry.  Floating-point expressions are evaluated in the reference's
// order so that sphere membership at R == rc resolves the same way.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <tuple>

#include "lcp_internal.h"

namespace lcp {

namespace {

constexpr double kPi = 3.14159265358979323846;

// Generation_ATV! (src/utils/Generation_ATV.jl:51-88): cell 0 is the home
// cell, then (i, j, k) in [-N, N]^3 with k fastest.
void gen_atv(int N, const double lat[3][3], std::vector<double>& atv, std::vector<int32_t>& ijk,
             std::vector<int32_t>& ratv) {
  const int n = 2 * N + 1;
  atv.assign((size_t)n * n * n * 3, 0.0);
  ijk.assign((size_t)n * n * n * 3, 0);
  ratv.assign((size_t)n * n * n, 0);
  int rn = 1;
  for (int i = -N; i <= N; ++i)
    for (int j = -N; j <= N; ++j)
      for (int k = -N; k <= N; ++k) {
        if (i == 0 && j == 0 && k == 0) {
          ratv[((size_t)(i + N) * n + (j + N)) * n + (k + N)] = 0;
          continue;
        }
        for (int c = 0; c < 3; ++c) atv[rn * 3 + c] = i * lat[0][c] + j * lat[1][c] + k * lat[2][c];
        ijk[rn * 3 + 0] = i;
        ijk[rn * 3 + 1] = j;
        ijk[rn * 3 + 2] = k;
        ratv[((size_t)(i + N) * n + (j + N)) * n + (k + N)] = rn;
        ++rn;
      }
}

inline bool neighbour_test(const double* g1, const double* g2, const double* t, double rcut, double* rout) {
  double dx = std::fabs(g1[0] - g2[0] - t[0]);
  double dy = std::fabs(g1[1] - g2[1] - t[1]);
  double dz = std::fabs(g1[2] - g2[2] - t[2]);
  if (dx <= rcut && dy <= rcut && dz <= rcut) {
    double r = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (r <= rcut) {
      *rout = r;
      return true;
    }
  }
  return false;
}

// Estimate_Trn_System (src/UCell.jl:573-608): total neighbour count.
int64_t count_neighbours(const UCell& u, const std::vector<double>& atv) {
  const int nc = (int)(atv.size() / 3);
  int64_t total = 0;
  double r;
  for (int a = 0; a < u.natom; ++a)
    for (int b = 0; b < u.natom; ++b) {
      const double rcut = u.cut[a] + u.cut[b];
      for (int rn = 0; rn < nc; ++rn) {
        if (a == b && rn == 0) continue;
        if (neighbour_test(&u.gxyz[a * 3], &u.gxyz[b * 3], &atv[rn * 3], rcut, &r)) ++total;
      }
    }
  return total;
}

void inv3(const double m[3][3], double out[3][3]) {
  double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
               m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
               m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  out[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
  out[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
  out[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
  out[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
  out[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
  out[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
  out[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
  out[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
  out[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
}

inline int floordiv(int a, int n) {
  int q = a / n;
  if ((a % n != 0) && ((a < 0) != (n < 0))) --q;
  return q;
}

struct AtomSphere {
  std::vector<int32_t> gl, cl;
  bool has_out_of_range = false;
  bool out_before_first_in = false;
  double last_c[3] = {0, 0, 0};
  bool any = false;
};

}  // namespace

// The grid-index box [nmin, nmax] that Calc_AtomsGrid scans for one atom
// (src/UCell.jl:333-364).
void atom_box(const UCell& u, int a, int nmin[3], int nmax[3]) {
  double gT[3][3], grec[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) gT[i][j] = u.glat[j][i];
  inv3(gT, grec);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) grec[i][j] *= 2 * kPi;
  static const int kindex[3][2] = {{1, 2}, {2, 0}, {0, 1}};
  const double Gx = u.gxyz[a * 3], Gy = u.gxyz[a * 3 + 1], Gz = u.gxyz[a * 3 + 2];
  const double* L = &u.lat[0][0];
  double rc5 = u.cut[a] + 0.5;
  for (int k = 0; k < 3; ++k) {
    int i = kindex[k][0], j = kindex[k][1];
    double vx = L[i * 3 + 1] * L[j * 3 + 2] - L[i * 3 + 2] * L[j * 3 + 1];
    double vy = L[i * 3 + 2] * L[j * 3 + 0] - L[i * 3 + 0] * L[j * 3 + 2];
    double vz = L[i * 3 + 0] * L[j * 3 + 1] - L[i * 3 + 1] * L[j * 3 + 0];
    double coef = 1.0 / std::sqrt(vx * vx + vy * vy + vz * vz);
    vx *= coef;
    vy *= coef;
    vz *= coef;
    double cx = Gx + rc5 * vx - u.origin[0], cy = Gy + rc5 * vy - u.origin[1], cz = Gz + rc5 * vz - u.origin[2];
    nmax[k] = (int)std::trunc((cx * grec[k][0] + cy * grec[k][1] + cz * grec[k][2]) * 0.5 / kPi);
    cx = Gx - rc5 * vx - u.origin[0];
    cy = Gy - rc5 * vy - u.origin[1];
    cz = Gz - rc5 * vz - u.origin[2];
    nmin[k] = (int)std::trunc((cx * grec[k][0] + cy * grec[k][1] + cz * grec[k][2]) * 0.5 / kPi);
    if (nmax[k] < nmin[k]) std::swap(nmin[k], nmax[k]);
  }
}

namespace {

// Calc_AtomsGrid for one atom (src/UCell.jl:333-400).  `carry` is the Cxyz
// left by the previous atom (Find_CGrids! keeps it across calls).
void atom_sphere(const UCell& u, int a, const double carry[3], AtomSphere& out) {
  const int N1 = u.ngrid[0], N2 = u.ngrid[1], N3 = u.ngrid[2];
  const int C = u.cpycell;
  const int n = 2 * C + 1;
  const double Gx = u.gxyz[a * 3], Gy = u.gxyz[a * 3 + 1], Gz = u.gxyz[a * 3 + 2];
  int nmin[3], nmax[3];
  atom_box(u, a, nmin, nmax);
  const double rcut = u.cut[a];
  double c[3] = {carry[0], carry[1], carry[2]};
  bool seen_in = false;
  std::vector<int32_t> gl, cl;
  for (int n1 = nmin[0]; n1 <= nmax[0]; ++n1)
    for (int n2 = nmin[1]; n2 <= nmax[1]; ++n2)
      for (int n3 = nmin[2]; n3 <= nmax[2]; ++n3) {
        int l1 = floordiv(n1, N1), l2 = floordiv(n2, N2), l3 = floordiv(n3, N3);
        int nn1 = n1 - l1 * N1, nn2 = n2 - l2 * N2, nn3 = n3 - l3 * N3;
        // Find_CGrids! checks the index shifted by one (src/utils/Find_CGrid.jl:7-11)
        int s1 = l1 + 1, s2 = l2 + 1, s3 = l3 + 1;
        int rn = 0;
        if (C < std::abs(s1) || C < std::abs(s2) || C < std::abs(s3)) {
          out.has_out_of_range = true;
          if (!seen_in) out.out_before_first_in = true;
        } else {
          seen_in = true;
          rn = u.ratv[((size_t)(C + s1 - 1) * n + (C + s2 - 1)) * n + (C + s3 - 1)];
          for (int d = 0; d < 3; ++d)
            c[d] = u.atv[rn * 3 + d] + nn1 * u.glat[0][d] + nn2 * u.glat[1][d] + nn3 * u.glat[2][d] + u.origin[d];
        }
        double dx = c[0] - Gx, dy = c[1] - Gy, dz = c[2] - Gz;
        double R = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (R <= rcut) {
          gl.push_back(nn1 * N2 * N3 + nn2 * N3 + nn3);
          cl.push_back(rn);
        }
        out.any = true;
      }
  out.last_c[0] = c[0];
  out.last_c[1] = c[1];
  out.last_c[2] = c[2];
  std::vector<int32_t> idx(gl.size());
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int32_t)i;
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t x, int32_t y) { return gl[x] < gl[y]; });
  out.gl.resize(gl.size());
  out.cl.resize(gl.size());
  for (size_t i = 0; i < idx.size(); ++i) {
    out.gl[i] = gl[idx[i]];
    out.cl[i] = cl[idx[i]];
  }
}

int hw_threads() {
  unsigned h = std::thread::hardware_concurrency();
  return h == 0 ? 4 : (int)std::min(h, 64u);
}

template <class F>
void parallel_for(int64_t n, F f) {
  int nt = (int)std::min<int64_t>(hw_threads(), std::max<int64_t>(n, 1));
  if (nt <= 1) {
    for (int64_t i = 0; i < n; ++i) f(i, 0);
    return;
  }
  std::atomic<int64_t> next(0);
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      for (;;) {
        int64_t i = next.fetch_add(1);
        if (i >= n) break;
        f(i, t);
      }
    });
  for (auto& x : th) x.join();
}

// Unrolled lattice coordinate of a sphere entry: grid index + cell * Ngrid.
inline void unrolled(const UCell& u, int32_t gn, int32_t cell, int& x, int& y, int& z) {
  const int N2 = u.ngrid[1], N3 = u.ngrid[2];
  int nn1 = gn / (N2 * N3);
  int nn2 = (gn - nn1 * N2 * N3) / N3;
  int nn3 = gn - nn1 * N2 * N3 - nn2 * N3;
  x = nn1 + u.atv_ijk[cell * 3 + 0] * u.ngrid[0];
  y = nn2 + u.atv_ijk[cell * 3 + 1] * u.ngrid[1];
  z = nn3 + u.atv_ijk[cell * 3 + 2] * N3;
}

// Dense lookup (unrolled coordinate -> index in the atom's sphere list).
struct SphereLUT {
  int lo[3] = {0, 0, 0}, ext[3] = {0, 0, 0};
  std::vector<int32_t> idx;
  void build(const UCell& u, int a) {
    int64_t s = u.sphere_off[a], e = u.sphere_off[a + 1];
    int mn[3] = {1 << 30, 1 << 30, 1 << 30}, mx[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int64_t k = s; k < e; ++k) {
      int p[3];
      unrolled(u, u.glist[k], u.clist[k], p[0], p[1], p[2]);
      for (int d = 0; d < 3; ++d) {
        mn[d] = std::min(mn[d], p[d]);
        mx[d] = std::max(mx[d], p[d]);
      }
    }
    if (e == s) {
      ext[0] = ext[1] = ext[2] = 0;
      idx.clear();
      return;
    }
    for (int d = 0; d < 3; ++d) {
      lo[d] = mn[d];
      ext[d] = mx[d] - mn[d] + 1;
    }
    idx.assign((size_t)ext[0] * ext[1] * ext[2], -1);
    for (int64_t k = s; k < e; ++k) {
      int p[3];
      unrolled(u, u.glist[k], u.clist[k], p[0], p[1], p[2]);
      idx[((size_t)(p[0] - lo[0]) * ext[1] + (p[1] - lo[1])) * ext[2] + (p[2] - lo[2])] = (int32_t)(k - s);
    }
  }
  inline int32_t find(int x, int y, int z) const {
    x -= lo[0];
    y -= lo[1];
    z -= lo[2];
    if (x < 0 || y < 0 || z < 0 || x >= ext[0] || y >= ext[1] || z >= ext[2]) return -1;
    return idx[((size_t)x * ext[1] + y) * ext[2] + z];
  }
};

// Calc_AtomOverlap_Grid for one pair (src/UCell.jl:439-512): for each point
// Nh of jatom's list, the entry of atom's list at the same physical point
// (same grid index, image cell = cell(Nh) + R), kept in Nh order.
void overlap_with_lut(const UCell& u, const SphereLUT& lut, int32_t pair, std::vector<int32_t>& g1,
                      std::vector<int32_t>& g2) {
  g1.clear();
  g2.clear();
  const int b = u.pair_jatom[pair];
  const int C = u.cpycell;
  const int r0 = u.atv_ijk[u.pair_cell[pair] * 3 + 0];
  const int r1 = u.atv_ijk[u.pair_cell[pair] * 3 + 1];
  const int r2 = u.atv_ijk[u.pair_cell[pair] * 3 + 2];
  int64_t s = u.sphere_off[b], e = u.sphere_off[b + 1];
  const int N2 = u.ngrid[1], N3 = u.ngrid[2];
  for (int64_t k = s; k < e; ++k) {
    int cell = u.clist[k];
    int l1 = u.atv_ijk[cell * 3 + 0] + r0, l2 = u.atv_ijk[cell * 3 + 1] + r1, l3 = u.atv_ijk[cell * 3 + 2] + r2;
    if (std::abs(l1) > C || std::abs(l2) > C || std::abs(l3) > C) continue;
    int gn = u.glist[k];
    int nn1 = gn / (N2 * N3);
    int nn2 = (gn - nn1 * N2 * N3) / N3;
    int nn3 = gn - nn1 * N2 * N3 - nn2 * N3;
    int32_t hit = lut.find(nn1 + l1 * u.ngrid[0], nn2 + l2 * N2, nn3 + l3 * N3);
    if (hit >= 0) {
      g1.push_back(hit);
      g2.push_back((int32_t)(k - s));
    }
  }
}

}  // namespace

void pair_overlap(const UCell& u, int32_t pair, std::vector<int32_t>& g1, std::vector<int32_t>& g2) {
  SphereLUT lut;
  lut.build(u, u.pair_atom[pair]);
  overlap_with_lut(u, lut, pair, g1, g2);
}

// Everything of UCell(...) but the sphere and overlap lists: checks, CpyCell
// and image cells, neighbour lists, the pair list with its DM/H block offsets
// and partners.
std::string build_ucell_head(UCell& u, int32_t nspin, const double* latvecs, int32_t natom,
                             const int32_t* atom2spe, const double* gxyz, const double* cut,
                             const int32_t* ngrid, const double* origin, const int32_t* numorbs) {
  if (natom <= 0) return "Natom must be positive";
  if (nspin != 1 && nspin != 2 && nspin != 4) return "Nspin must be 1, 2 or 4";
  for (int d = 0; d < 3; ++d)
    if (ngrid[d] <= 0) return "Ngrid entries must be positive";
  u.nspin = nspin;
  u.natom = natom;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) u.lat[i][j] = latvecs[i * 3 + j];
  for (int d = 0; d < 3; ++d) {
    u.ngrid[d] = ngrid[d];
    u.origin[d] = origin ? origin[d] : 0.0;
    for (int c = 0; c < 3; ++c) u.glat[d][c] = u.lat[d][c] / ngrid[d];
  }
  u.atom2spe.assign(atom2spe, atom2spe + natom);
  u.gxyz.assign(gxyz, gxyz + natom * 3);
  u.cut.assign(cut, cut + natom);
  u.numorbs.assign(natom, 0);
  if (numorbs)
    for (int a = 0; a < natom; ++a) {
      if (numorbs[a] < 0) return "Total_NumOrbs must be >= 0";
      u.numorbs[a] = numorbs[a];
    }
  for (int a = 0; a < natom; ++a)
    if (!(u.cut[a] > 0)) return "Atoms_Cut1 must be positive";
  double det = u.lat[0][0] * (u.lat[1][1] * u.lat[2][2] - u.lat[1][2] * u.lat[2][1]) -
               u.lat[0][1] * (u.lat[1][0] * u.lat[2][2] - u.lat[1][2] * u.lat[2][0]) +
               u.lat[0][2] * (u.lat[1][0] * u.lat[2][1] - u.lat[1][1] * u.lat[2][0]);
  if (det == 0.0 || !std::isfinite(det)) return "Latvecs is singular";
  u.gridvol = std::fabs(det) / ((double)ngrid[0] * ngrid[1] * ngrid[2]);

  // Get_FNAN (src/UCell.jl:520-556)
  int cpy = 0, count = 1, po = 0;
  int64_t tf = 0;
  while (po == 0 && count < 7) {
    ++cpy;
    std::vector<double> atv;
    std::vector<int32_t> ijk, ratv;
    gen_atv(cpy, u.lat, atv, ijk, ratv);
    int64_t prev = tf;
    tf = count_neighbours(u, atv);
    if (tf == prev) po = 1;
    ++count;
  }
  if (count == 7 || po == 0) return "please check Get_FNAN";
  u.cpycell = cpy;
  gen_atv(cpy, u.lat, u.atv, u.atv_ijk, u.ratv);
  u.ncell = (int32_t)(u.atv.size() / 3);

  // Trn_System (src/UCell.jl:612-672)
  u.fnan.assign(natom, 0);
  u.natn.assign(natom, {});
  u.ncn.assign(natom, {});
  double r;
  for (int a = 0; a < natom; ++a) {
    u.natn[a].push_back(a + 1);
    u.ncn[a].push_back(0);
    for (int b = 0; b < natom; ++b) {
      const double rcut = u.cut[a] + u.cut[b];
      for (int rn = 0; rn < u.ncell; ++rn) {
        if (a == b && rn == 0) continue;
        if (neighbour_test(&u.gxyz[a * 3], &u.gxyz[b * 3], &u.atv[rn * 3], rcut, &r)) {
          u.natn[a].push_back(b + 1);
          u.ncn[a].push_back(rn);
        }
      }
    }
    u.fnan[a] = (int32_t)u.natn[a].size() - 1;
  }

  // flattened pair list and DM/H block offsets (src/UCell.jl:82-128)
  u.pair_atom.clear();
  u.pair_jatom.clear();
  u.pair_cell.clear();
  u.block_off.clear();
  int64_t off = 0;
  std::vector<int32_t> first_pair(natom + 1, 0);
  for (int a = 0; a < natom; ++a) {
    first_pair[a] = (int32_t)u.pair_atom.size();
    for (int k = 0; k <= u.fnan[a]; ++k) {
      u.pair_atom.push_back(a);
      u.pair_jatom.push_back(u.natn[a][k] - 1);
      u.pair_cell.push_back(u.ncn[a][k]);
      u.block_off.push_back(off);
      off += (int64_t)u.numorbs[a] * u.numorbs[u.natn[a][k] - 1];
    }
  }
  first_pair[natom] = (int32_t)u.pair_atom.size();
  u.nloop = (int32_t)u.pair_atom.size();
  u.total_hsize = off;

  // partner (j, i, -R) of every pair
  const int C = cpy, n = 2 * C + 1;
  u.partner.assign(u.nloop, -1);
  for (int a = 0; a < natom; ++a) {
    std::map<std::pair<int, int>, int> where;
    for (int k = 0; k <= u.fnan[a]; ++k) where[{u.natn[a][k] - 1, u.ncn[a][k]}] = first_pair[a] + k;
    for (int p = 0; p < u.nloop; ++p) {
      if (u.pair_jatom[p] != a) continue;
      int c = u.pair_cell[p];
      int mi = -u.atv_ijk[c * 3], mj = -u.atv_ijk[c * 3 + 1], mk = -u.atv_ijk[c * 3 + 2];
      int negc = u.ratv[((size_t)(mi + C) * n + (mj + C)) * n + (mk + C)];
      auto it = where.find({u.pair_atom[p], negc});
      if (it == where.end()) return "neighbour list is not symmetric";
      u.partner[p] = it->second;
    }
  }
  for (int p = 0; p < u.nloop; ++p)
    if (u.partner[p] < 0) return "neighbour list is not symmetric";

  // the kept orientation of each folded pair
  u.uniq_pair.clear();
  for (int p = 0; p < u.nloop; ++p)
    if (p <= u.partner[p]) u.uniq_pair.push_back(p);
  return "";
}

// Calc_AtomsGrid (src/UCell.jl:297-411): the sphere lists.
void build_spheres_host(UCell& u) {
  const int natom = u.natom;
  // Atoms are independent unless an image cell falls outside +-CpyCell before
  // the first in-range point, when the previous atom's stale Cxyz matters;
  // then redo sequentially.
  std::vector<AtomSphere> sph(natom);
  const double zero3[3] = {0, 0, 0};
  parallel_for(natom, [&](int64_t a, int) { atom_sphere(u, (int)a, zero3, sph[a]); });
  bool need_seq = false;
  for (int a = 1; a < natom; ++a)
    if (sph[a].out_before_first_in) need_seq = true;
  if (need_seq) {
    double carry[3] = {0, 0, 0};
    for (int a = 0; a < natom; ++a) {
      AtomSphere s;
      atom_sphere(u, a, carry, s);
      if (s.any)
        for (int d = 0; d < 3; ++d) carry[d] = s.last_c[d];
      sph[a] = std::move(s);
    }
  }
  u.sphere_off.assign(natom + 1, 0);
  for (int a = 0; a < natom; ++a) u.sphere_off[a + 1] = u.sphere_off[a] + (int64_t)sph[a].gl.size();
  u.glist.resize(u.sphere_off[natom]);
  u.clist.resize(u.sphere_off[natom]);
  for (int a = 0; a < natom; ++a) {
    std::copy(sph[a].gl.begin(), sph[a].gl.end(), u.glist.begin() + u.sphere_off[a]);
    std::copy(sph[a].cl.begin(), sph[a].cl.end(), u.clist.begin() + u.sphere_off[a]);
  }
  sph.clear();
}

// Calc_AtomOverlap_Grid (src/UCell.jl:425-516): the exact overlap lists of the
// kept orientation of each folded pair, and NumOLG of every pair.
void build_overlaps_host(UCell& u) {
  const int natom = u.natom;
  const int64_t nu = (int64_t)u.uniq_pair.size();
  std::vector<std::vector<int32_t>> ug1(nu), ug2(nu);
  // group folded pairs by their atom so that one lookup table serves a group
  std::vector<std::vector<int64_t>> by_atom(natom);
  for (int64_t q = 0; q < nu; ++q) by_atom[u.pair_atom[u.uniq_pair[q]]].push_back(q);
  parallel_for(natom, [&](int64_t a, int) {
    if (by_atom[a].empty()) return;
    SphereLUT lut;
    lut.build(u, (int)a);
    for (int64_t q : by_atom[a]) overlap_with_lut(u, lut, u.uniq_pair[q], ug1[q], ug2[q]);
  });
  u.uniq_off.assign(nu + 1, 0);
  for (int64_t q = 0; q < nu; ++q) u.uniq_off[q + 1] = u.uniq_off[q] + (int64_t)ug1[q].size();
  u.uniq_g1.resize(u.uniq_off[nu]);
  u.uniq_g2.resize(u.uniq_off[nu]);
  u.numolg.assign(u.nloop, 0);
  for (int64_t q = 0; q < nu; ++q) {
    std::copy(ug1[q].begin(), ug1[q].end(), u.uniq_g1.begin() + u.uniq_off[q]);
    std::copy(ug2[q].begin(), ug2[q].end(), u.uniq_g2.begin() + u.uniq_off[q]);
    int p = u.uniq_pair[q];
    u.numolg[p] = (int64_t)ug1[q].size();
    u.numolg[u.partner[p]] = (int64_t)ug1[q].size();
  }
}

std::string build_ucell(UCell& u, int32_t nspin, const double* latvecs, int32_t natom,
                        const int32_t* atom2spe, const double* gxyz, const double* cut,
                        const int32_t* ngrid, const double* origin, const int32_t* numorbs) {
  std::string e = build_ucell_head(u, nspin, latvecs, natom, atom2spe, gxyz, cut, ngrid, origin, numorbs);
  if (!e.empty()) return e;
  build_spheres_host(u);
  build_overlaps_host(u);
  return "";
}

// Predicted cost (arbitrary units) of grid bricks of shape bd: each brick
// costs kBrick, each (brick, 16-orbital sub-image) block kImage and each pair
// of sub-images of a brick kPair (the tensor-core passes are one K step per
// image pair and window, plus per-image table traffic).  The blocks of an atom
// are estimated as the volume of its cutoff sphere grown by a brick (Steiner
// formula for a box) over the average brick volume.
double brick_shape_cost(const UCell& u, const int32_t* bd) {
  constexpr double kBrick = 2.0, kImage = 1.0, kPair = 0.125, kPi = 3.14159265358979323846;
  double L[3], nbr = 1.0, vcell;
  for (int d = 0; d < 3; ++d) {
    const double len = std::sqrt(u.lat[d][0] * u.lat[d][0] + u.lat[d][1] * u.lat[d][1] + u.lat[d][2] * u.lat[d][2]);
    L[d] = len / u.ngrid[d] * bd[d];
    nbr *= (double)((u.ngrid[d] + bd[d] - 1) / bd[d]);
  }
  vcell = std::fabs(u.lat[0][0] * (u.lat[1][1] * u.lat[2][2] - u.lat[1][2] * u.lat[2][1]) -
                    u.lat[0][1] * (u.lat[1][0] * u.lat[2][2] - u.lat[1][2] * u.lat[2][0]) +
                    u.lat[0][2] * (u.lat[1][0] * u.lat[2][1] - u.lat[1][1] * u.lat[2][0]));
  const double veff = vcell / nbr;
  const double s2 = L[0] * L[1] + L[1] * L[2] + L[0] * L[2], s1 = L[0] + L[1] + L[2], v3 = L[0] * L[1] * L[2];
  double blocks = 0.0;
  for (int a = 0; a < u.natom; ++a) {
    const int nch = (u.numorbs[a] + 15) / 16;
    const double r = u.cut[a];
    blocks += nch * (v3 + 2 * r * s2 + kPi * r * r * s1 + 4.0 / 3.0 * kPi * r * r * r) / veff;
  }
  const double m = blocks / nbr;
  return nbr * (kBrick + kImage * m + kPair * m * m);
}

std::vector<std::array<int32_t, 3>> brick_shape_candidates(const UCell& u, std::vector<double>* costs) {
  std::vector<std::pair<double, std::array<int32_t, 3>>> all;
  for (int b0 = 1; b0 <= 8; ++b0)
    for (int b1 = 1; b1 <= 8; ++b1)
      for (int b2 = 1; b2 <= 8; ++b2) {
        const int prod = b0 * b1 * b2;
        if (prod > 128 || prod < 16 || b0 > u.ngrid[0] || b1 > u.ngrid[1] || b2 > u.ngrid[2]) continue;
        const int32_t bd[3] = {b0, b1, b2};
        all.push_back({brick_shape_cost(u, bd), {b0, b1, b2}});
      }
  std::stable_sort(all.begin(), all.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
  std::vector<std::array<int32_t, 3>> out;
  if (costs) costs->clear();
  for (auto& c : all) {
    out.push_back(c.second);
    if (costs) costs->push_back(c.first);
  }
  return out;
}

std::string build_bricks(const UCell& u, Bricks& b, const int32_t* shape) {
  if (!shape || shape[0] <= 0) {
    // the predicted best shape whose bricks stay within kMaxBrickImages
    // sub-images (a smaller brick touches fewer atom images)
    // (after a shape overflows, only shapes of fewer points are tried)
    const auto cand = brick_shape_candidates(u, nullptr);
    if (cand.empty()) return "no brick shape fits the grid";
    std::string err;
    int limit = 129, tries = 0;
    for (size_t i = 0; i < cand.size() && tries < 12; ++i) {
      const int prod = cand[i][0] * cand[i][1] * cand[i][2];
      if (prod >= limit) continue;
      ++tries;
      err = build_bricks(u, b, cand[i].data());
      if (!err.empty() || b.max_images <= kMaxBrickImages) return err;
      limit = prod;
    }
    return err;
  }
  int best[3];
  for (int d = 0; d < 3; ++d) {
    if (shape[d] < 1 || shape[d] > u.ngrid[d]) return "brick shape out of range";
    best[d] = shape[d];
  }
  if (best[0] * best[1] * best[2] > 128) return "a brick holds at most 128 points";
  // bricks tile each period of the grid from 0; the last brick of an axis is
  // ragged when the brick side does not divide Ngrid
  for (int d = 0; d < 3; ++d) {
    b.bdim[d] = best[d];
    b.nb[d] = (u.ngrid[d] + best[d] - 1) / best[d];
  }
  b.npts = best[0] * best[1] * best[2];
  b.nbricks = (int64_t)b.nb[0] * b.nb[1] * b.nb[2];
  const int64_t npoints = u.sphere_off.empty() ? 0 : u.sphere_off.back();
  b.point_code.assign(npoints, 0);
  b.block_atom.clear();
  // orbital chunks: an atom with NO orbitals is ceil(NO/16) sub-images of 16
  std::vector<int32_t> nch(u.natom);
  for (int a = 0; a < u.natom; ++a) nch[a] = (u.numorbs[a] + 15) / 16;
  struct Img {
    int32_t atom, block, r0, r1, r2;
  };
  std::vector<std::vector<Img>> per_brick(b.nbricks);
  for (int a = 0; a < u.natom; ++a) {
    if (nch[a] == 0) continue;  // no orbitals: no blocks
    std::map<std::tuple<int, int, int>, int32_t> blocks;
    for (int64_t k = u.sphere_off[a]; k < u.sphere_off[a + 1]; ++k) {
      int x, y, z;
      unrolled(u, u.glist[k], u.clist[k], x, y, z);
      // period R and home brick h per axis: c = R * nb + h
      int l0, l1, l2, c0, c1, c2;
      {
        const int xs[3] = {x, y, z};
        int ls[3], cs[3];
        for (int d = 0; d < 3; ++d) {
          const int R = floordiv(xs[d], u.ngrid[d]);
          const int g = xs[d] - R * u.ngrid[d];
          const int h = g / b.bdim[d];
          ls[d] = g - h * b.bdim[d];
          cs[d] = R * b.nb[d] + h;
        }
        l0 = ls[0], l1 = ls[1], l2 = ls[2], c0 = cs[0], c1 = cs[1], c2 = cs[2];
      }
      auto key = std::make_tuple(c0, c1, c2);
      auto it = blocks.find(key);
      int32_t blk;
      if (it == blocks.end()) {
        blk = (int32_t)b.block_atom.size();  // the chunks' blocks are blk .. blk + nch - 1
        for (int c = 0; c < nch[a]; ++c) b.block_atom.push_back(a);
        blocks.emplace(key, blk);
        int h0 = c0 - floordiv(c0, b.nb[0]) * b.nb[0];
        int h1 = c1 - floordiv(c1, b.nb[1]) * b.nb[1];
        int h2 = c2 - floordiv(c2, b.nb[2]) * b.nb[2];
        int64_t hb = ((int64_t)h0 * b.nb[1] + h1) * b.nb[2] + h2;
        per_brick[hb].push_back({a, blk, floordiv(c0, b.nb[0]), floordiv(c1, b.nb[1]), floordiv(c2, b.nb[2])});
      } else {
        blk = it->second;
      }
      const int slot = (l0 * b.bdim[1] + l1) * b.bdim[2] + l2;
      b.point_code[k] = blk * 128 + slot;
    }
  }
  b.nblocks = (int64_t)b.block_atom.size();
  // ordered pair of (atom, jatom, cell)
  std::map<std::tuple<int, int, int>, int32_t> pair_of;
  for (int p = 0; p < u.nloop; ++p) pair_of[{u.pair_atom[p], u.pair_jatom[p], u.pair_cell[p]}] = p;
  // sub-pairs: (pair, row chunk, column chunk), numbered pair-major
  b.sub_off.assign(u.nloop + 1, 0);
  for (int p = 0; p < u.nloop; ++p)
    b.sub_off[p + 1] = b.sub_off[p] + (int64_t)nch[u.pair_atom[p]] * nch[u.pair_jatom[p]];
  b.nsub = b.sub_off[u.nloop];
  b.sub_pair.resize(b.nsub);
  b.sub_chunks.resize(b.nsub);
  for (int p = 0; p < u.nloop; ++p)
    for (int ca = 0; ca < nch[u.pair_atom[p]]; ++ca)
      for (int cb = 0; cb < nch[u.pair_jatom[p]]; ++cb) {
        const int64_t sp = b.sub_off[p] + (int64_t)ca * nch[u.pair_jatom[p]] + cb;
        b.sub_pair[sp] = p;
        b.sub_chunks[sp] = (ca << 8) | cb;
      }
  const int C = u.cpycell, n = 2 * C + 1;
  b.img_off.assign(b.nbricks + 1, 0);
  b.tab_off.assign(b.nbricks + 1, 0);
  b.img_block.clear();
  b.img_atom.clear();
  b.tab_pair.clear();
  b.max_images = 0;
  for (int64_t hb = 0; hb < b.nbricks; ++hb) {
    auto& v = per_brick[hb];
    std::sort(v.begin(), v.end(), [](const Img& x, const Img& y) {
      return std::make_tuple(x.atom, x.r0, x.r1, x.r2) < std::make_tuple(y.atom, y.r0, y.r1, y.r2);
    });
    // sub-images: each image's chunks, consecutive
    std::vector<int32_t> img_of, chunk_of;
    for (int s = 0; s < (int)v.size(); ++s)
      for (int c = 0; c < nch[v[s].atom]; ++c) {
        b.img_block.push_back(v[s].block + c);
        b.img_atom.push_back(v[s].atom);
        img_of.push_back(s);
        chunk_of.push_back(c);
      }
    const int m = (int)img_of.size();
    b.max_images = std::max(b.max_images, m);
    b.img_off[hb + 1] = (int64_t)b.img_block.size();
    // image s = atom shifted by -R_s; pair (atom_s, atom_t, R_s - R_t); the
    // sub-image pair (s, ca), (t, cb) is that pair's sub-pair (ca, cb)
    for (int si = 0; si < m; ++si)
      for (int ti = 0; ti < m; ++ti) {
        const Img& vs = v[img_of[si]];
        const Img& vt = v[img_of[ti]];
        int d0 = vs.r0 - vt.r0, d1 = vs.r1 - vt.r1, d2 = vs.r2 - vt.r2;
        int32_t sub = -1;
        if (std::abs(d0) <= C && std::abs(d1) <= C && std::abs(d2) <= C) {
          int cell = u.ratv[((size_t)(d0 + C) * n + (d1 + C)) * n + (d2 + C)];
          auto it = pair_of.find({vs.atom, vt.atom, cell});
          if (it != pair_of.end())
            sub = (int32_t)(b.sub_off[it->second] + (int64_t)chunk_of[si] * nch[vt.atom] + chunk_of[ti]);
        }
        b.tab_pair.push_back(sub);
      }
    b.tab_off[hb + 1] = (int64_t)b.tab_pair.size();
  }
  // Number the blocks in image order: every block is an image of exactly one
  // home brick, so a brick's images become consecutive blocks and a window of
  // them is one contiguous range of the tables.
  {
    std::vector<int32_t> perm(b.nblocks, -1);
    for (size_t i = 0; i < b.img_block.size(); ++i) perm[b.img_block[i]] = (int32_t)i;
    std::vector<int32_t> atom_of(b.nblocks);
    for (int64_t k = 0; k < b.nblocks; ++k) atom_of[perm[k]] = b.block_atom[k];
    b.block_atom.swap(atom_of);
    for (auto& c : b.point_code) c = perm[c >> 7] * 128 + (c & 127);
    for (size_t i = 0; i < b.img_block.size(); ++i) b.img_block[i] = (int32_t)i;
  }
  // grid-H slots: (s <= t) sub-image pairs of each brick that are neighbour
  // pairs.  Each feeds one 16 x 16 sub-block (ca, cb) of its folded pair's
  // kept orientation: directly when its pair is the kept one, transposed as
  // (cb, ca) when it is the partner; a self pair's slot between two different
  // chunks of the same image also feeds the transposed sub-block.
  std::vector<int32_t> fold(u.nloop, -1);
  for (size_t q = 0; q < u.uniq_pair.size(); ++q) {
    fold[u.uniq_pair[q]] = (int32_t)q;
    fold[u.partner[u.uniq_pair[q]]] = (int32_t)q;
  }
  b.sb_off.assign(u.uniq_pair.size() + 1, 0);
  for (size_t q = 0; q < u.uniq_pair.size(); ++q) {
    const int p0 = u.uniq_pair[q];
    b.sb_off[q + 1] = b.sb_off[q] + (int64_t)nch[u.pair_atom[p0]] * nch[u.pair_jatom[p0]];
  }
  const int64_t nsb = b.sb_off.back();
  b.sb_fold.resize(nsb);
  b.sb_chunks.resize(nsb);
  for (size_t q = 0; q < u.uniq_pair.size(); ++q) {
    const int p0 = u.uniq_pair[q];
    for (int ca = 0; ca < nch[u.pair_atom[p0]]; ++ca)
      for (int cb = 0; cb < nch[u.pair_jatom[p0]]; ++cb) {
        const int64_t k = b.sb_off[q] + (int64_t)ca * nch[u.pair_jatom[p0]] + cb;
        b.sb_fold[k] = (int32_t)q;
        b.sb_chunks[k] = (ca << 8) | cb;
      }
  }
  b.tab_slot.assign(b.tab_pair.size(), -1);
  b.slot_base.assign(b.nbricks + 1, 0);
  std::vector<std::vector<int64_t>> per_sb(nsb);
  int64_t gslot = 0;
  for (int64_t hb = 0; hb < b.nbricks; ++hb) {
    const int m = (int)(b.img_off[hb + 1] - b.img_off[hb]);
    const int64_t t0 = b.tab_off[hb];
    b.slot_base[hb] = gslot;
    int local = 0;
    for (int s = 0; s < m; ++s)
      for (int t = s; t < m; ++t) {
        const int32_t sp = b.tab_pair[t0 + s * m + t];
        if (sp < 0) continue;
        b.tab_slot[t0 + s * m + t] = local++;
        const int32_t p = b.sub_pair[sp];
        const int ca = b.sub_chunks[sp] >> 8, cb = b.sub_chunks[sp] & 255;
        const int32_t q = fold[p];
        const int p0 = u.uniq_pair[q];
        const int ncj = nch[u.pair_jatom[p0]];
        if (p == p0) {
          per_sb[b.sb_off[q] + (int64_t)ca * ncj + cb].push_back(gslot * 2);
          if (u.partner[p0] == p0 && ca != cb) per_sb[b.sb_off[q] + (int64_t)cb * ncj + ca].push_back(gslot * 2 + 1);
        } else {
          per_sb[b.sb_off[q] + (int64_t)cb * ncj + ca].push_back(gslot * 2 + 1);
        }
        ++gslot;
      }
  }
  b.slot_base[b.nbricks] = gslot;
  // The reduction visits the sub-blocks longest first (stable, so the order is
  // fixed): their partial counts range from a few to thousands (self pairs),
  // and a long one started last would run alone at the end of the launch.
  // Each sub-block's own sum keeps its order, so H is the same bits.
  std::vector<int64_t> order(nsb);
  for (int64_t q = 0; q < nsb; ++q) order[q] = q;
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t x, int64_t y) { return per_sb[x].size() > per_sb[y].size(); });
  std::vector<int32_t> fold_o(nsb), chunks_o(nsb);
  b.red_off.assign(nsb + 1, 0);
  b.red_slot.clear();
  b.red_slot.reserve(gslot);
  for (int64_t k = 0; k < nsb; ++k) {
    const int64_t q = order[k];
    fold_o[k] = b.sb_fold[q];
    chunks_o[k] = b.sb_chunks[q];
    b.red_slot.insert(b.red_slot.end(), per_sb[q].begin(), per_sb[q].end());
    b.red_off[k + 1] = (int64_t)b.red_slot.size();
  }
  b.sb_fold.swap(fold_o);
  b.sb_chunks.swap(chunks_o);
  return "";
}

// Row q of inv(M), M[p][q] = x_p^i2 y_p^j2 z_p^k2 with q = 9 i2 + 3 j2 + k2 and
// p = 9 (i1+1) + 3 (j1+1) + (k1+1), holds the coefficient of monomial q of
// the fit as weights on the 27 values; rows 9, 3, 1 (the reference's 10, 4, 2)
// are the x, y and z monomials, i.e. the gradient at the centre.  Gauss-Jordan
// elimination with partial pivoting on [M | I].
bool calc_diff_coef(const double gtv[3][3], double out[81]) {
  constexpr int N = 27;
  std::vector<double> a((size_t)N * 2 * N, 0.0);
  auto A = [&](int r, int c) -> double& { return a[(size_t)r * 2 * N + c]; };
  int p = 0;
  for (int i1 = -1; i1 <= 1; ++i1)
    for (int j1 = -1; j1 <= 1; ++j1)
      for (int k1 = -1; k1 <= 1; ++k1, ++p) {
        double r[3];
        for (int d = 0; d < 3; ++d) r[d] = i1 * gtv[0][d] + j1 * gtv[1][d] + k1 * gtv[2][d];
        int q = 0;
        for (int i2 = 0; i2 <= 2; ++i2)
          for (int j2 = 0; j2 <= 2; ++j2)
            for (int k2 = 0; k2 <= 2; ++k2, ++q) {
              double m = 1.0;
              for (int e = 0; e < i2; ++e) m *= r[0];
              double my = 1.0;
              for (int e = 0; e < j2; ++e) my *= r[1];
              double mz = 1.0;
              for (int e = 0; e < k2; ++e) mz *= r[2];
              A(p, q) = m * my * mz;
            }
        A(p, N + p) = 1.0;
      }
  for (int c = 0; c < N; ++c) {
    int piv = c;
    for (int r = c + 1; r < N; ++r)
      if (std::fabs(A(r, c)) > std::fabs(A(piv, c))) piv = r;
    if (!(std::fabs(A(piv, c)) > 0.0)) return false;
    if (piv != c)
      for (int k = 0; k < 2 * N; ++k) std::swap(A(c, k), A(piv, k));
    const double inv = 1.0 / A(c, c);
    for (int k = 0; k < 2 * N; ++k) A(c, k) *= inv;
    for (int r = 0; r < N; ++r) {
      if (r == c) continue;
      const double f = A(r, c);
      if (f == 0.0) continue;
      for (int k = 0; k < 2 * N; ++k) A(r, k) -= f * A(c, k);
    }
  }
  const int rows[3] = {9, 3, 1};
  for (int d = 0; d < 3; ++d)
    for (int k = 0; k < N; ++k) out[d * N + k] = A(rows[d], N + k);
  return true;
}

}  // namespace lcp
