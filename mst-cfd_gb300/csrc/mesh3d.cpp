// 3D solver mesh: corrected geometry and device layout (see mesh3d.hpp).
// Compile with -ffp-contract=off.
#include "mesh3d.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>

namespace mst {
namespace {

inline double dot3(const double* a, const double* b) {
  double s = a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}

int kind3(int type, int c1) {
  switch (type) {
    case kInterior: return c1 >= 0 ? kKindInterior : kKindNone;
    case kInlet: return kKindInlet;
    case kWall: return kKindWall;
    case kSymmetry: return kKindSymmetry;
    case kOutlet: return kKindOutlet;
    default: return kKindNone;
  }
}

// 21-bit spread for a 3D Morton key
uint64_t spread3(uint32_t v) {
  uint64_t x = v & 0x1FFFFF;
  x = (x | (x << 32)) & 0x1F00000000FFFFull;
  x = (x | (x << 16)) & 0x1F0000FF0000FFull;
  x = (x | (x << 8)) & 0x100F00F00F00F00Full;
  x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

}  // namespace

int build_solver3d(const HostMesh3D& h, const std::vector<double>& c1_shift, SolverMesh3D* s,
                   std::string* err) {
  const int nF = h.n_faces, nC = h.n_cells;
  const bool per = !c1_shift.empty();
  if (per && c1_shift.size() != 3 * (size_t)nF) {
    *err = "c1_shift must hold 3 numbers per face";
    return kEInval;
  }
  SolverMesh3D& m = *s;
  m = SolverMesh3D{};
  m.n_cells = nC;
  m.n_faces = nF;
  m.face_cells.assign(2 * (size_t)nF, -1);
  m.face_kind.assign(nF, kKindNone);
  m.face_ctr.assign(3 * (size_t)nF, 0.0);
  m.face_dir.assign(3 * (size_t)nF, 0.0);
  m.r0.assign(3 * (size_t)nF, 0.0);
  m.r1.assign(3 * (size_t)nF, 0.0);
  m.eta.assign(nF, 1.0);
  m.cell_ctr.assign(3 * (size_t)nC, 0.0);
  m.cell_vol.assign(nC, 0.0);
  m.cell_ptr.assign(nC + 1, 0);
  for (int f = 0; f < nF; ++f) {
    const int c0 = h.face_cells[2 * (size_t)f], c1 = h.face_cells[2 * (size_t)f + 1];
    const int b = h.face_ptr[f], n = h.face_ptr[f + 1] - b;
    if (c0 < 0 || c0 >= nC || c1 >= nC || (n != 3 && n != 4)) {
      *err = "3D solver: face with bad cells or a node count other than 3 or 4";
      return kEMesh;
    }
    m.face_cells[2 * (size_t)f] = c0;
    m.face_cells[2 * (size_t)f + 1] = c1;
    m.face_kind[f] = kind3(h.face_type[f], c1);
    const double* p0 = &h.node_xyz[3 * (size_t)h.face_nodes[b]];
    const double* p1 = &h.node_xyz[3 * (size_t)h.face_nodes[b + 1]];
    const double* p2 = &h.node_xyz[3 * (size_t)h.face_nodes[b + 2]];
    for (int d = 0; d < 3; ++d) {
      double sm = p0[d];
      sm += p1[d];
      sm += p2[d];
      if (n == 4) sm += h.node_xyz[3 * (size_t)h.face_nodes[b + 3] + d];
      m.face_ctr[3 * (size_t)f + d] = sm / (double)n;
    }
    double a[3], bb[3];
    if (n == 3) {
      for (int d = 0; d < 3; ++d) {
        a[d] = p1[d] - p0[d];
        bb[d] = p2[d] - p0[d];
      }
    } else {
      const double* p3 = &h.node_xyz[3 * (size_t)h.face_nodes[b + 3]];
      for (int d = 0; d < 3; ++d) {
        a[d] = p2[d] - p0[d];
        bb[d] = p3[d] - p1[d];
      }
    }
    double* dv = &m.face_dir[3 * (size_t)f];
    dv[0] = 0.5 * (a[1] * bb[2] - a[2] * bb[1]);
    dv[1] = 0.5 * (a[2] * bb[0] - a[0] * bb[2]);
    dv[2] = 0.5 * (a[0] * bb[1] - a[1] * bb[0]);
    m.cell_ptr[c0 + 1]++;
    if (c1 >= 0) m.cell_ptr[c1 + 1]++;
  }
  for (int c = 0; c < nC; ++c) {
    if (m.cell_ptr[c + 1] == 0) {
      *err = "3D solver: cell without faces";
      return kEMesh;
    }
    m.cell_ptr[c + 1] += m.cell_ptr[c];
  }
  const int tot = m.cell_ptr[nC];
  m.cell_faces.assign(tot, 0);
  m.cell_nb.assign(tot, -1);
  {
    std::vector<int> fill(m.cell_ptr.begin(), m.cell_ptr.end() - 1);
    for (int f = 0; f < nF; ++f) {
      const int c0 = m.face_cells[2 * (size_t)f], c1 = m.face_cells[2 * (size_t)f + 1];
      m.cell_faces[fill[c0]] = f;
      m.cell_nb[fill[c0]++] = c1;
      if (c1 >= 0) {
        m.cell_faces[fill[c1]] = f;
        m.cell_nb[fill[c1]++] = c0;
      }
    }
  }
  for (int c = 0; c < nC; ++c) {
    const int kb = m.cell_ptr[c], ke = m.cell_ptr[c + 1];
    double sm[3] = {0.0, 0.0, 0.0};
    for (int k = kb; k < ke; ++k) {
      const int f = m.cell_faces[k];
      const bool own = m.face_cells[2 * (size_t)f] == c;
      for (int d = 0; d < 3; ++d) {
        double x = m.face_ctr[3 * (size_t)f + d];
        if (!own && per) x = x - c1_shift[3 * (size_t)f + d];
        sm[d] += x;
      }
    }
    for (int d = 0; d < 3; ++d) m.cell_ctr[3 * (size_t)c + d] = sm[d] / (double)(ke - kb);
  }
  for (int f = 0; f < nF; ++f) {
    const int c0 = m.face_cells[2 * (size_t)f], c1 = m.face_cells[2 * (size_t)f + 1];
    double t[3];
    for (int d = 0; d < 3; ++d)
      t[d] = m.face_ctr[3 * (size_t)f + d] - m.cell_ctr[3 * (size_t)c0 + d];
    double* dv = &m.face_dir[3 * (size_t)f];
    if (dot3(dv, t) < 0.0)
      for (int d = 0; d < 3; ++d) dv[d] = -dv[d];
    for (int d = 0; d < 3; ++d) m.r0[3 * (size_t)f + d] = t[d];
    if (c1 >= 0) {
      for (int d = 0; d < 3; ++d) {
        double x = m.face_ctr[3 * (size_t)f + d];
        if (per) x = x - c1_shift[3 * (size_t)f + d];
        m.r1[3 * (size_t)f + d] = x - m.cell_ctr[3 * (size_t)c1 + d];
      }
      const double n0 = std::sqrt(dot3(&m.r0[3 * (size_t)f], &m.r0[3 * (size_t)f]));
      const double n1 = std::sqrt(dot3(&m.r1[3 * (size_t)f], &m.r1[3 * (size_t)f]));
      m.eta[f] = n1 / (n0 + n1);
    }
  }
  m.cell_dir.assign(3 * (size_t)tot, 0.0);
  m.cell_w.assign(2 * (size_t)tot, 0.0);
  for (int c = 0; c < nC; ++c) {
    double v = 0.0;
    for (int k = m.cell_ptr[c]; k < m.cell_ptr[c + 1]; ++k) {
      const int f = m.cell_faces[k];
      const bool own = m.face_cells[2 * (size_t)f] == c;
      const double* r = own ? &m.r0[3 * (size_t)f] : &m.r1[3 * (size_t)f];
      double* cd = &m.cell_dir[3 * (size_t)k];
      for (int d = 0; d < 3; ++d)
        cd[d] = own ? m.face_dir[3 * (size_t)f + d] : -m.face_dir[3 * (size_t)f + d];
      m.cell_w[2 * (size_t)k] = own ? m.eta[f] : 1.0 - m.eta[f];
      m.cell_w[2 * (size_t)k + 1] = own ? 1.0 - m.eta[f] : m.eta[f];
      v += dot3(r, cd);
    }
    m.cell_vol[c] = v / 3.0;
    if (!(m.cell_vol[c] > 0.0)) {
      *err = "3D solver: cell of non-positive volume";
      return kEMesh;
    }
  }
  return kOk;
}

int build_layout3d(const SolverMesh3D& m, DevLayout3D* L, std::string* err) {
  const int nC = m.n_cells, nF = m.n_faces;
  L->n_cells = nC;
  L->n_faces = nF;
  L->cell_iperm.resize(nC);
  std::iota(L->cell_iperm.begin(), L->cell_iperm.end(), 0);
  if (nC > kTileCells) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int c = 0; c < nC; ++c)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], m.cell_ctr[3 * (size_t)c + d]);
        hi[d] = std::max(hi[d], m.cell_ctr[3 * (size_t)c + d]);
      }
    std::vector<uint64_t> key(nC);
    for (int c = 0; c < nC; ++c) {
      uint64_t k = 0;
      for (int d = 0; d < 3; ++d) {
        const double span = hi[d] - lo[d];
        double u = span > 0 ? (m.cell_ctr[3 * (size_t)c + d] - lo[d]) / span : 0.0;
        if (!(u >= 0)) u = 0;
        const uint32_t qd = (uint32_t)std::min(2097151.0, std::floor(u * 2097152.0));
        k |= spread3(qd) << d;
      }
      key[c] = k;
    }
    std::stable_sort(L->cell_iperm.begin(), L->cell_iperm.end(),
                     [&](int a, int b) { return key[a] < key[b]; });
  }
  L->cell_perm.assign(nC, 0);
  for (int i = 0; i < nC; ++i) L->cell_perm[L->cell_iperm[i]] = i;
  const int nT = (nC + kTileCells - 1) / kTileCells;
  L->n_tiles = nT;
  std::vector<int> owner(nF);
  for (int f = 0; f < nF; ++f) {
    const int a = L->cell_perm[m.face_cells[2 * (size_t)f]];
    const int c1 = m.face_cells[2 * (size_t)f + 1];
    const int b = c1 >= 0 ? L->cell_perm[c1] : a;
    owner[f] = std::min(a, b) / kTileCells;
  }
  // device faces grouped by owner tile (counting sort, file order within)
  L->t_own_ptr.assign(nT + 1, 0);
  for (int f = 0; f < nF; ++f) L->t_own_ptr[owner[f] + 1]++;
  for (int t = 0; t < nT; ++t) L->t_own_ptr[t + 1] += L->t_own_ptr[t];
  L->face_perm.assign(nF, 0);
  std::vector<int> face_iperm(nF);
  {
    std::vector<int> fill(L->t_own_ptr.begin(), L->t_own_ptr.end() - 1);
    for (int f = 0; f < nF; ++f) {
      const int df = fill[owner[f]]++;
      L->face_perm[f] = df;
      face_iperm[df] = f;
    }
  }
  // borrowed faces: cut faces owned by the other tile, ascending device id
  L->t_bor_ptr.assign(nT + 1, 0);
  for (int f = 0; f < nF; ++f) {
    const int c1 = m.face_cells[2 * (size_t)f + 1];
    if (c1 < 0) continue;
    const int ta = L->cell_perm[m.face_cells[2 * (size_t)f]] / kTileCells;
    const int tb = L->cell_perm[c1] / kTileCells;
    if (ta != tb) L->t_bor_ptr[std::max(ta, tb) + 1]++;
  }
  for (int t = 0; t < nT; ++t) L->t_bor_ptr[t + 1] += L->t_bor_ptr[t];
  L->t_bor.assign(L->t_bor_ptr[nT], 0);
  {
    std::vector<int> fill(L->t_bor_ptr.begin(), L->t_bor_ptr.end() - 1);
    for (int df = 0; df < nF; ++df) {  // device order: each list ascends
      const int f = face_iperm[df];
      const int c1 = m.face_cells[2 * (size_t)f + 1];
      if (c1 < 0) continue;
      const int ta = L->cell_perm[m.face_cells[2 * (size_t)f]] / kTileCells;
      const int tb = L->cell_perm[c1] / kTileCells;
      if (ta != tb) L->t_bor[fill[std::max(ta, tb)]++] = df;
    }
  }
  L->max_tile_faces = 0;
  for (int t = 0; t < nT; ++t)
    L->max_tile_faces =
        std::max(L->max_tile_faces, (L->t_own_ptr[t + 1] - L->t_own_ptr[t]) +
                                        (L->t_bor_ptr[t + 1] - L->t_bor_ptr[t]));
  L->f_c0c1.assign(2 * (size_t)nF, -1);
  L->f_info.assign(nF, 0);
  L->f_dir.assign(3 * (size_t)nF, 0.0);
  L->f_r0.assign(3 * (size_t)nF, 0.0);
  L->f_r1.assign(3 * (size_t)nF, 0.0);
  L->f_eta.assign(nF, 1.0);
  for (int df = 0; df < nF; ++df) {
    const int f = face_iperm[df];
    const int c0 = m.face_cells[2 * (size_t)f], c1 = m.face_cells[2 * (size_t)f + 1];
    L->f_c0c1[2 * (size_t)df] = L->cell_perm[c0];
    L->f_c0c1[2 * (size_t)df + 1] = c1 >= 0 ? L->cell_perm[c1] : -1;
    int info = m.face_kind[f];
    for (int d = 0; d < 3; ++d) {
      if (m.face_dir[3 * (size_t)f + d] >= 0.0) info |= 1 << (kInfo3Flag + d);
      L->f_dir[3 * (size_t)df + d] = m.face_dir[3 * (size_t)f + d];
      L->f_r0[3 * (size_t)df + d] = m.r0[3 * (size_t)f + d];
      L->f_r1[3 * (size_t)df + d] = m.r1[3 * (size_t)f + d];
    }
    L->f_info[df] = info;
    L->f_eta[df] = m.eta[f];
  }
  L->c_vol.assign(nC, 0.0);
  L->c_ptr.assign(nC + 1, 0);
  for (int dc = 0; dc < nC; ++dc) {
    const int c = L->cell_iperm[dc];
    L->c_vol[dc] = m.cell_vol[c];
    L->c_ptr[dc + 1] = L->c_ptr[dc] + (m.cell_ptr[c + 1] - m.cell_ptr[c]);
  }
  const int tot = L->c_ptr[nC];
  L->cf_slot.assign(tot, 0);
  L->cf_nb.assign(tot, -1);
  L->cf_w.assign(2 * (size_t)tot, 0.0);
  L->cf_dir.assign(3 * (size_t)tot, 0.0);
  for (int t = 0; t < nT; ++t) {
    const int ob = L->t_own_ptr[t], oe = L->t_own_ptr[t + 1], n_own = oe - ob;
    const int* bb = L->t_bor.data() + L->t_bor_ptr[t];
    const int* be = L->t_bor.data() + L->t_bor_ptr[t + 1];
    const int cb = t * kTileCells, ce = std::min(nC, cb + kTileCells);
    for (int dc = cb; dc < ce; ++dc) {
      const int c = L->cell_iperm[dc];
      for (int j = 0; j < m.cell_ptr[c + 1] - m.cell_ptr[c]; ++j) {
        const int k = m.cell_ptr[c] + j, dk = L->c_ptr[dc] + j;
        const int f = m.cell_faces[k], df = L->face_perm[f];
        int slot;
        if (df >= ob && df < oe) {
          slot = df - ob;
        } else {
          const int* p = std::lower_bound(bb, be, df);
          if (p == be || *p != df) {
            *err = "internal: face missing from its tile";
            return kEInval;
          }
          slot = n_own + (int)(p - bb);
        }
        const bool own = m.face_cells[2 * (size_t)f] == c;
        L->cf_slot[dk] = (slot << 1) | (own ? 0 : 1);
        const int nb = m.cell_nb[k];
        L->cf_nb[dk] = nb >= 0 ? L->cell_perm[nb] : -1;
        L->cf_w[2 * (size_t)dk] = m.cell_w[2 * (size_t)k];
        L->cf_w[2 * (size_t)dk + 1] = m.cell_w[2 * (size_t)k + 1];
        for (int d = 0; d < 3; ++d) L->cf_dir[3 * (size_t)dk + d] = m.cell_dir[3 * (size_t)k + d];
      }
    }
  }
  return kOk;
}

}  // namespace mst
