// Host mesh front end; see mesh.hpp.  Compile with -ffp-contract=off.
#include "mesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>

namespace mst {
namespace {

// hexStringToInt (work/FUNCTION.cpp:41-55): lower-case hex digits; any other
// character keeps its digit position but adds nothing.
int hex_value(const std::string& s) {
  int v = 0;
  for (char c : s) {
    int w = 0;
    if (c >= 'a' && c <= 'f') w = c - 'a' + 10;
    else if (c >= '0' && c <= '9') w = c - '0';
    v = v * 16 + w;
  }
  return v;
}

// Tokens separated by single spaces (getline(stream, tok, ' ')).
std::vector<std::string> split_spaces(const std::string& s) {
  std::vector<std::string> t;
  size_t b = 0;
  for (;;) {
    size_t e = s.find(' ', b);
    if (e == std::string::npos) {
      t.push_back(s.substr(b));
      break;
    }
    t.push_back(s.substr(b, e - b));
    b = e + 1;
  }
  return t;
}

// Text between the second '(' and the next ')' (betweenSecBrackets,
// FUNCTION.cpp:64-72); empty if there is no second '('.
bool second_bracket(const std::string& s, std::string* out) {
  size_t a = s.find('(');
  if (a == std::string::npos) return false;
  size_t b = s.find('(', a + 1);
  if (b == std::string::npos) return false;
  size_t c = s.find(')', b + 1);
  *out = s.substr(b + 1, c == std::string::npos ? std::string::npos : c - b - 1);
  return true;
}

inline double nrm(double a, double b) { return std::sqrt(a * a + b * b); }

}  // namespace

int read_msh(const std::string& path, HostMesh* m, std::string* err) {
  std::ifstream in(path, std::ios::binary);
  if (!in) {
    *err = "cannot open " + path;
    return kEInval;
  }
  std::string text((std::istreambuf_iterator<char>(in)),
                   std::istreambuf_iterator<char>());
  // Header lines start with '(' or ')'; everything else is data, in order.
  // '\r' is dropped (the reference was run in Windows text mode).
  std::vector<std::string> hdr, dat;
  dat.emplace_back();  // the reference's data stream begins with "\n"
  size_t b = 0;
  while (b < text.size()) {
    size_t e = text.find('\n', b);
    if (e == std::string::npos) e = text.size();
    std::string line = text.substr(b, e - b);
    while (!line.empty() && line.back() == '\r') line.pop_back();
    if (!line.empty() && (line[0] == '(' || line[0] == ')')) hdr.push_back(line);
    else dat.push_back(line);
    b = e + 1;
  }
  // Totals (10 (0 1 N 0 D)) (12 (0 ...)) (13 (0 ...)).
  int nN = -1, nC = -1, nF = -1;
  for (const auto& s : hdr) {
    std::string br;
    if (s.size() < 3 || s[1] != '1' || !second_bracket(s, &br) || br.empty() ||
        br[0] != '0')
      continue;
    auto t = split_spaces(br);
    if (t.size() < 3) continue;
    int v = hex_value(t[2]);
    if (s[2] == '0') nN = v;
    if (s[2] == '2') nC = v;
    if (s[2] == '3') nF = v;
  }
  if (nN <= 0 || nC <= 0 || nF <= 0) {
    *err = "missing node/cell/face totals";
    return kEMesh;
  }
  m->n_nodes = nN;
  m->n_cells = nC;
  m->n_faces = nF;
  m->node_xy.assign(2 * (size_t)nN, 0.0);
  m->face_nodes.assign(2 * (size_t)nF, -1);
  m->face_cells.assign(2 * (size_t)nF, -1);
  m->face_type.assign(nF, 0);
  m->zone.clear();
  m->c1_shift.clear();
  m->n_int_faces = 0;
  size_t di = 0;
  int flag_node = 0, flag_face = 0;
  for (const auto& s : hdr) {
    std::string br;
    if (s.size() < 3 || s[1] != '1' || !second_bracket(s, &br) || br.empty() ||
        br[0] == '0')
      continue;
    if (s[2] == '0') {
      // node section: one data line is consumed first (MshBlock.cpp:192)
      ++di;
      for (; flag_node < nN; ++flag_node) {
        if (di >= dat.size()) {
          *err = "node section truncated";
          return kEMesh;
        }
        auto t = split_spaces(dat[di++]);
        if (t.size() < 2 || t[0].empty() || t[1].empty()) {
          *err = "bad node line";
          return kEMesh;
        }
        for (int d = 0; d < 2; ++d)
          m->node_xy[2 * flag_node + d] = std::strtod(t[d].c_str(), nullptr);
      }
    } else if (s[2] == '3') {
      auto t = split_spaces(br);
      if (t.size() < 5) {
        *err = "bad face zone header";
        return kEMesh;
      }
      int zid = hex_value(t[0]), st = hex_value(t[1]), en = hex_value(t[2]),
          ty = hex_value(t[3]), nn = hex_value(t[4]);
      if (nn != 2 || en > nF || st != flag_face + 1) {
        *err = "unsupported face zone (mixed elements, gaps or 3D)";
        return kEMesh;
      }
      m->zone.insert(m->zone.end(), {zid, st, en, ty});
      if (ty == kInterior) m->n_int_faces = en;
      for (; flag_face < en; ++flag_face) {
        if (di >= dat.size()) {
          *err = "face section truncated";
          return kEMesh;
        }
        auto tk = split_spaces(dat[di++]);
        size_t need = (ty == kInterior) ? 4 : 3;
        if (tk.size() < need) {
          *err = "bad face line";
          return kEMesh;
        }
        int n0 = hex_value(tk[0]) - 1, n1 = hex_value(tk[1]) - 1;
        int c0 = hex_value(tk[2]) - 1;
        int c1 = (ty == kInterior) ? hex_value(tk[3]) - 1 : -1;
        if (n0 < 0 || n0 >= nN || n1 < 0 || n1 >= nN || c0 < 0 || c0 >= nC ||
            (ty == kInterior && (c1 < 0 || c1 >= nC))) {
          *err = "face references a missing node or cell";
          return kEMesh;
        }
        m->face_nodes[2 * flag_face] = n0;
        m->face_nodes[2 * flag_face + 1] = n1;
        m->face_cells[2 * flag_face] = c0;
        m->face_cells[2 * flag_face + 1] = c1;
        m->face_type[flag_face] = ty;
      }
    }
  }
  if (flag_node != nN || flag_face != nF || m->zone.empty()) {
    *err = "node or face sections incomplete";
    return kEMesh;
  }
  return build_geometry(m, err);
}

int build_from_arrays(int n_nodes, const double* node_xy, int n_cells,
                      int n_faces, const int* face_nodes,
                      const int* face_cells, int n_zones, const int* zones,
                      const double* c1_shift, HostMesh* m, std::string* err) {
  if (n_nodes <= 0 || n_cells <= 0 || n_faces <= 0 || n_zones <= 0 ||
      !node_xy || !face_nodes || !face_cells || !zones) {
    *err = "empty mesh description";
    return kEInval;
  }
  m->n_nodes = n_nodes;
  m->n_cells = n_cells;
  m->n_faces = n_faces;
  m->node_xy.assign(node_xy, node_xy + 2 * (size_t)n_nodes);
  m->face_nodes.assign(face_nodes, face_nodes + 2 * (size_t)n_faces);
  m->face_cells.assign(face_cells, face_cells + 2 * (size_t)n_faces);
  m->zone.assign(zones, zones + 4 * (size_t)n_zones);
  m->face_type.assign(n_faces, 0);
  m->n_int_faces = 0;
  int expect = 1;
  for (int z = 0; z < n_zones; ++z) {
    int st = zones[4 * z + 1], en = zones[4 * z + 2], ty = zones[4 * z + 3];
    if (st != expect || en < st - 1 || en > n_faces) {
      *err = "zones must cover the faces contiguously and in order";
      return kEInval;
    }
    expect = en + 1;
    if (ty == kInterior) m->n_int_faces = en;
    for (int i = st - 1; i < en; ++i) {
      m->face_type[i] = ty;
      if (ty != kInterior) m->face_cells[2 * i + 1] = -1;
    }
  }
  if (expect != n_faces + 1) {
    *err = "zones do not cover every face";
    return kEInval;
  }
  for (int i = 0; i < n_faces; ++i) {
    int n0 = face_nodes[2 * i], n1 = face_nodes[2 * i + 1];
    int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
    if (n0 < 0 || n0 >= n_nodes || n1 < 0 || n1 >= n_nodes || c0 < 0 ||
        c0 >= n_cells || c1 >= n_cells ||
        (m->face_type[i] == kInterior && c1 < 0)) {
      *err = "face references a missing node or cell";
      return kEInval;
    }
  }
  if (c1_shift) {
    m->c1_shift.assign(c1_shift, c1_shift + 2 * (size_t)n_faces);
  } else {
    m->c1_shift.clear();
  }
  return build_geometry(m, err);
}

int build_geometry(HostMesh* m, std::string* err) {
  const int nC = m->n_cells, nF = m->n_faces, nI = m->n_int_faces;
  const bool per = m->periodic();
  auto shift = [&](int f, int d) { return per ? m->c1_shift[2 * f + d] : 0.0; };
  // cell -> face lists in face order (c0, then c1, of each face), and the
  // neighbour cell per cell-face (the cell itself on boundary faces)
  m->cell_ptr.assign(nC + 1, 0);
  for (int i = 0; i < nF; ++i) {
    m->cell_ptr[m->face_cells[2 * i] + 1]++;
    if (m->face_cells[2 * i + 1] >= 0) m->cell_ptr[m->face_cells[2 * i + 1] + 1]++;
  }
  for (int c = 0; c < nC; ++c) m->cell_ptr[c + 1] += m->cell_ptr[c];
  const int tot = m->cell_ptr[nC];
  m->cell_faces.assign(tot, 0);
  m->cell_nb.assign(tot, 0);
  {
    std::vector<int> fill(nC, 0);
    for (int i = 0; i < nF; ++i) {
      int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
      int k0 = m->cell_ptr[c0] + fill[c0]++;
      m->cell_faces[k0] = i;
      m->cell_nb[k0] = (c1 >= 0) ? c1 : c0;
      if (c1 >= 0) {
        int k1 = m->cell_ptr[c1] + fill[c1]++;
        m->cell_faces[k1] = i;
        m->cell_nb[k1] = c0;
      }
    }
  }
  // Face::setCenter (Face.cpp:8-19)
  m->face_ctr.assign(2 * (size_t)nF, 0.0);
  m->face_dir.assign(2 * (size_t)nF, 0.0);
  m->face_area.assign(nF, 0.0);
  for (int i = 0; i < nF; ++i) {
    const double* a = &m->node_xy[2 * m->face_nodes[2 * i]];
    const double* b = &m->node_xy[2 * m->face_nodes[2 * i + 1]];
    for (int d = 0; d < 2; ++d) {
      double s = 0.0;
      s += a[d];
      s += b[d];
      m->face_ctr[2 * i + d] = s / 2.0;
    }
    double f0 = a[0] - b[0], f1 = a[1] - b[1];
    m->face_area[i] = nrm(f0, f1);
    m->face_dir[2 * i] = -f1;
    m->face_dir[2 * i + 1] = f0;
  }
  // face centre seen from each cell (periodic images live in c1's frame)
  m->cell_face_ctr.assign(2 * (size_t)tot, 0.0);
  for (int c = 0; c < nC; ++c)
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      int f = m->cell_faces[k];
      bool as_c1 = m->face_cells[2 * f] != c;
      for (int d = 0; d < 2; ++d)
        m->cell_face_ctr[2 * k + d] =
            as_c1 ? m->face_ctr[2 * f + d] - shift(f, d) : m->face_ctr[2 * f + d];
    }
  // Cell::setCenter / setVolume (Cell.cpp:6-50)
  m->cell_ctr.assign(2 * (size_t)nC, 0.0);
  m->cell_vol.assign(nC, 0.0);
  for (int c = 0; c < nC; ++c) {
    const int b = m->cell_ptr[c], n = m->cell_ptr[c + 1] - b;
    for (int d = 0; d < 2; ++d) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += m->cell_face_ctr[2 * (b + k) + d];
      m->cell_ctr[2 * c + d] = s / (double)n;
    }
    auto len = [&](int k) {
      int f = m->cell_faces[b + k];
      return nrm(m->face_dir[2 * f], m->face_dir[2 * f + 1]);
    };
    auto fc = [&](int k, int d) { return m->cell_face_ctr[2 * (b + k) + d]; };
    double vol;
    if (n == 3) {
      double l0 = len(0), l1 = len(1), l2 = len(2);
      double s = 0.5 * (l0 + l1 + l2);
      vol = std::sqrt(s * (s - l0) * (s - l1) * (s - l2));
    } else if (n == 4) {
      double v1x = fc(0, 0) - fc(1, 0), v1y = fc(0, 1) - fc(1, 1);
      double v2x = fc(2, 0) - fc(3, 0), v2y = fc(2, 1) - fc(3, 1);
      int a0, a1, b0, b1;
      double mid;
      if (std::fabs(v1x * v2y - v2x * v1y) < 1e-7) {
        mid = 2 * nrm(fc(0, 0) - fc(1, 0), fc(0, 1) - fc(1, 1));
        a0 = 0, a1 = 1, b0 = 2, b1 = 3;
      } else {
        mid = 2 * nrm(fc(0, 0) - fc(2, 0), fc(0, 1) - fc(2, 1));
        a0 = 0, a1 = 2, b0 = 1, b1 = 3;
      }
      double la0 = len(a0), la1 = len(a1), lb0 = len(b0), lb1 = len(b1);
      double s = 0.5 * (la0 + la1 + mid);
      vol = std::sqrt(s * (s - la0) * (s - la1) * (s - mid));
      double s2 = 0.5 * (lb0 + lb1 + mid);
      vol += std::sqrt(s2 * (s2 - lb0) * (s2 - lb1) * (s2 - mid));
    } else {
      *err = "cell with " + std::to_string(n) +
             " faces: the 2D path handles triangles and quads";
      return kEMesh;
    }
    m->cell_vol[c] = vol;
  }
  // orientation flags (MshBlock.cpp:281-305) and the geometric flags
  m->face_dac.assign(nF, 1);
  m->face_flag.assign(2 * (size_t)nF, 0);
  m->face_flag_geo.assign(2 * (size_t)nF, 0);
  for (int i = 0; i < nF; ++i) {
    int c0 = m->face_cells[2 * i];
    const double* dv = &m->face_dir[2 * i];
    double t = dv[0] * (m->face_ctr[2 * i] - m->cell_ctr[2 * c0]);
    t += dv[1] * (m->face_ctr[2 * i + 1] - m->cell_ctr[2 * c0 + 1]);
    if (t < 0) {
      m->face_dac[i] = -1;
      for (int d = 0; d < 2; ++d) m->face_flag[2 * i + d] = (-1.0 * dv[d] >= 0);
    } else {
      m->face_dac[i] = 1;
      for (int d = 0; d < 2; ++d) m->face_flag[2 * i + d] = !(1.0 * dv[d] >= 0);
    }
    // c0 is the left state along axis d when its outward normal points +d
    for (int d = 0; d < 2; ++d)
      m->face_flag_geo[2 * i + d] = (m->face_dac[i] * dv[d] >= 0);
  }
  // directOfNbFaces (:307-318)
  m->cell_dof.assign(2 * (size_t)tot, 0.0);
  for (int c = 0; c < nC; ++c)
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      int f = m->cell_faces[k];
      double s = (double)((m->face_cells[2 * f] == c) ? m->face_dac[f] : -m->face_dac[f]);
      m->cell_dof[2 * k] = s * m->face_dir[2 * f];
      m->cell_dof[2 * k + 1] = s * m->face_dir[2 * f + 1];
    }
  // eta0 (Face.cpp:62-69), eta0C (MshBlock.cpp:323-334)
  m->face_eta0.assign(nF, 1.0);
  for (int i = 0; i < nF; ++i) {
    int c0 = m->face_cells[2 * i], c1 = m->face_cells[2 * i + 1];
    if (c1 < 0) continue;
    const double* fcn = &m->face_ctr[2 * i];
    double x1 = m->cell_ctr[2 * c1] + shift(i, 0), y1 = m->cell_ctr[2 * c1 + 1] + shift(i, 1);
    double n1 = nrm(x1 - fcn[0], y1 - fcn[1]);
    double n0 = nrm(m->cell_ctr[2 * c0] - fcn[0], m->cell_ctr[2 * c0 + 1] - fcn[1]);
    m->face_eta0[i] = n1 / (n0 + n1);
  }
  m->cell_eta0c.assign(tot, 0.0);
  for (int c = 0; c < nC; ++c)
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      int f = m->cell_faces[k];
      m->cell_eta0c[k] = (m->face_cells[2 * f] == c) ? m->face_eta0[f] : 1 - m->face_eta0[f];
    }
  // boundary cell lists (:370-406)
  std::vector<uint8_t> flag(nC, 0);
  m->bond1.clear();
  m->bond2.clear();
  m->inner.clear();
  for (int i = 0; i < nF; ++i)
    if (m->face_type[i] != kInterior) {
      int c0 = m->face_cells[2 * i];
      if (!flag[c0]) {
        m->bond1.push_back(c0);
        flag[c0] = 1;
      }
    }
  for (int c : std::vector<int>(m->bond1))
    for (int k = m->cell_ptr[c]; k < m->cell_ptr[c + 1]; ++k) {
      int nb = m->cell_nb[k];
      if (!flag[nb]) {
        m->bond2.push_back(nb);
        flag[nb] = 1;
      }
    }
  for (int c = 0; c < nC; ++c)
    if (!flag[c]) m->inner.push_back(c);
  (void)nI;
  return kOk;
}

// ---------------------------------------------------------------------------
// device layout
// ---------------------------------------------------------------------------
namespace {
uint64_t spread_bits(uint32_t v) {
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
  x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
  x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}
int face_kind(int type) {
  switch (type) {
    case kInterior: return kKindInterior;
    case kInlet: return kKindInlet;
    case kWall: return kKindWall;
    case kSymmetry: return kKindSymmetry;
    case kOutlet: return kKindOutlet;
    default: return kKindNone;
  }
}
}  // namespace

int build_layout(const HostMesh& m, bool renumber, DevLayout* L,
                 std::string* err) {
  const int nC = m.n_cells, nF = m.n_faces, nI = m.n_int_faces;
  L->n_cells = nC;
  L->n_faces = nF;
  // cell order: Morton curve of the centroids (stable in file order)
  L->cell_iperm.resize(nC);
  std::iota(L->cell_iperm.begin(), L->cell_iperm.end(), 0);
  if (renumber && nC > kTileCells) {
    // one Morton curve per case (a single mesh is one case); cases keep
    // their order, so the device cells of a case are contiguous
    std::vector<int> seg = m.case_cells;
    if (seg.empty()) seg = {0, nC};
    std::vector<uint64_t> key(nC);
    for (size_t s = 0; s + 1 < seg.size(); ++s) {
      double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300};
      for (int c = seg[s]; c < seg[s + 1]; ++c)
        for (int d = 0; d < 2; ++d) {
          lo[d] = std::min(lo[d], m.cell_ctr[2 * c + d]);
          hi[d] = std::max(hi[d], m.cell_ctr[2 * c + d]);
        }
      for (int c = seg[s]; c < seg[s + 1]; ++c) {
        uint32_t q[2];
        for (int d = 0; d < 2; ++d) {
          double span = hi[d] - lo[d];
          double u = span > 0 ? (m.cell_ctr[2 * c + d] - lo[d]) / span : 0.0;
          if (!(u >= 0)) u = 0;  // NaN centroids go first
          q[d] = (uint32_t)std::min(65535.0, std::floor(u * 65536.0));
        }
        key[c] = ((uint64_t)s << 32) | spread_bits(q[0]) | (spread_bits(q[1]) << 1);
      }
    }
    std::stable_sort(L->cell_iperm.begin(), L->cell_iperm.end(),
                     [&](int a, int b) { return key[a] < key[b]; });
  }
  L->cell_perm.assign(nC, 0);
  for (int i = 0; i < nC; ++i) L->cell_perm[L->cell_iperm[i]] = i;
  const int nT = (nC + kTileCells - 1) / kTileCells;
  L->n_tiles = nT;
  auto tile_of = [&](int dev_cell) { return dev_cell / kTileCells; };
  // face order: by owner tile (tile of the lower device cell), file order
  std::vector<int> owner(nF);
  for (int i = 0; i < nF; ++i) {
    int a = L->cell_perm[m.face_cells[2 * i]];
    int c1 = m.face_cells[2 * i + 1];
    int b = c1 >= 0 ? L->cell_perm[c1] : a;
    owner[i] = tile_of(std::min(a, b));
  }
  L->face_iperm.resize(nF);
  std::iota(L->face_iperm.begin(), L->face_iperm.end(), 0);
  std::stable_sort(L->face_iperm.begin(), L->face_iperm.end(),
                   [&](int a, int b) { return owner[a] < owner[b]; });
  L->face_perm.assign(nF, 0);
  for (int i = 0; i < nF; ++i) L->face_perm[L->face_iperm[i]] = i;
  L->t_own_ptr.assign(nT + 1, 0);
  for (int i = 0; i < nF; ++i) L->t_own_ptr[owner[i] + 1]++;
  for (int t = 0; t < nT; ++t) L->t_own_ptr[t + 1] += L->t_own_ptr[t];
  // borrowed faces: cut faces owned by the other tile
  std::vector<std::vector<int>> bor(nT);
  for (int i = 0; i < nF; ++i) {
    int c1 = m.face_cells[2 * i + 1];
    if (c1 < 0) continue;
    int ta = tile_of(L->cell_perm[m.face_cells[2 * i]]);
    int tb = tile_of(L->cell_perm[c1]);
    if (ta != tb) bor[std::max(ta, tb)].push_back(L->face_perm[i]);
  }
  L->t_bor_ptr.assign(nT + 1, 0);
  L->t_bor.clear();
  L->max_tile_faces = 0;
  for (int t = 0; t < nT; ++t) {
    std::sort(bor[t].begin(), bor[t].end());
    L->t_bor.insert(L->t_bor.end(), bor[t].begin(), bor[t].end());
    L->t_bor_ptr[t + 1] = (int)L->t_bor.size();
    int n = (L->t_own_ptr[t + 1] - L->t_own_ptr[t]) + (int)bor[t].size();
    L->max_tile_faces = std::max(L->max_tile_faces, n);
  }
  // face arrays
  L->f_c0c1.assign(2 * (size_t)nF, -1);
  L->f_info.assign(nF, 0);
  L->f_dir.assign(2 * (size_t)nF, 0.0);
  L->f_r0.assign(2 * (size_t)nF, 0.0);
  L->f_r1.assign(2 * (size_t)nF, 0.0);
  const bool per = m.periodic();
  for (int df = 0; df < nF; ++df) {
    int f = L->face_iperm[df];
    int c0 = m.face_cells[2 * f], c1 = m.face_cells[2 * f + 1];
    L->f_c0c1[2 * df] = L->cell_perm[c0];
    L->f_c0c1[2 * df + 1] = c1 >= 0 ? L->cell_perm[c1] : -1;
    int info = face_kind(m.face_type[f]);
    if (!m.face_case.empty()) info |= m.face_case[f] << kInfoCaseShift;
    for (int d = 0; d < 2; ++d) {
      if (m.face_flag[2 * f + d]) info |= 1 << (kInfoFlagRef + d);
      if (m.face_flag_geo[2 * f + d]) info |= 1 << (kInfoFlagGeo + d);
    }
    L->f_info[df] = info;
    for (int d = 0; d < 2; ++d) {
      L->f_dir[2 * df + d] = m.face_dir[2 * f + d];
      // reconstruction offsets, x_f - x_c, as RhoSolver.cpp:250 evaluates
      L->f_r0[2 * df + d] = m.face_ctr[2 * f + d] - m.cell_ctr[2 * c0 + d];
      if (c1 >= 0) {
        double xf = per ? m.face_ctr[2 * f + d] - m.c1_shift[2 * f + d]
                        : m.face_ctr[2 * f + d];
        L->f_r1[2 * df + d] = xf - m.cell_ctr[2 * c1 + d];
      }
    }
  }
  // cells
  L->c_vol.assign(nC, 0.0);
  L->c_ptr.assign(nC + 1, 0);
  for (int dc = 0; dc < nC; ++dc) {
    int c = L->cell_iperm[dc];
    L->c_vol[dc] = m.cell_vol[c];
    L->c_ptr[dc + 1] = L->c_ptr[dc] + (m.cell_ptr[c + 1] - m.cell_ptr[c]);
  }
  const int tot = L->c_ptr[nC];
  L->cf_face.assign(tot, 0);
  L->cf_slot.assign(tot, 0);
  L->cf_nb.assign(tot, 0);
  L->cf_nb_fix.assign(tot, 0);
  L->cf_w.assign(2 * (size_t)tot, 0.0);
  for (int t = 0; t < nT; ++t) {
    // tile-local slot of every face the tile touches
    const int ob = L->t_own_ptr[t], oe = L->t_own_ptr[t + 1];
    const int n_own = oe - ob;
    auto slot_of = [&](int df) -> int {
      if (df >= ob && df < oe) return df - ob;
      const int* b = L->t_bor.data() + L->t_bor_ptr[t];
      const int* e = L->t_bor.data() + L->t_bor_ptr[t + 1];
      const int* p = std::lower_bound(b, e, df);
      if (p == e || *p != df) return -1;
      return n_own + (int)(p - b);
    };
    const int cb = t * kTileCells, ce = std::min(nC, cb + kTileCells);
    for (int dc = cb; dc < ce; ++dc) {
      int c = L->cell_iperm[dc];
      for (int j = 0; j < m.cell_ptr[c + 1] - m.cell_ptr[c]; ++j) {
        int k = m.cell_ptr[c] + j, dk = L->c_ptr[dc] + j;
        int f = m.cell_faces[k], df = L->face_perm[f];
        bool is_c0 = m.face_cells[2 * f] == c;
        bool neg = (is_c0 ? m.face_dac[f] : -m.face_dac[f]) < 0;
        L->cf_face[dk] = neg ? ~df : df;
        int s = slot_of(df);
        if (s < 0) {
          *err = "internal: face missing from its tile";
          return kEInval;
        }
        L->cf_slot[dk] = (s << 1) | (neg ? 1 : 0);
        int nb = L->cell_perm[m.cell_nb[k]];
        // face values for the gradient (RhoSolver.cpp:434-440): interpolated
        // on interior faces, the c0 value from the first boundary-loop face
        auto mode_for = [&](int first_copy) {
          if (f < first_copy && m.face_cells[2 * f + 1] >= 0) return (int)kFvInterp;
          return is_c0 ? (int)kFvSelf : (int)kFvNb;
        };
        int quirk_first = nI > 0 ? nI - 1 : 0;
        L->cf_nb[dk] = nb | (mode_for(quirk_first) << kFvShift);
        L->cf_nb_fix[dk] = nb | (mode_for(nI) << kFvShift);
        double e = m.face_eta0[f];
        // self weight and neighbour weight, each the same rounded number as
        // the reference's eta0 and (1 - eta0)
        L->cf_w[2 * dk] = is_c0 ? e : 1 - e;
        L->cf_w[2 * dk + 1] = is_c0 ? 1 - e : e;
      }
    }
  }
  // fused-pass tables: halo cells per tile, local cell indices per face slot
  // and per cell-face
  {
    std::vector<std::vector<int>> halo(nT);
    for (int i = 0; i < nF; ++i) {
      const int c1 = m.face_cells[2 * i + 1];
      if (c1 < 0) continue;
      const int a = L->cell_perm[m.face_cells[2 * i]], b = L->cell_perm[c1];
      const int ta = tile_of(a), tb = tile_of(b);
      if (ta == tb) continue;
      halo[ta].push_back(b);
      halo[tb].push_back(a);
    }
    L->t_halo_ptr.assign(nT + 1, 0);
    L->t_halo.clear();
    L->max_halo = 0;
    for (int t = 0; t < nT; ++t) {
      auto& h = halo[t];
      std::sort(h.begin(), h.end());
      h.erase(std::unique(h.begin(), h.end()), h.end());
      L->t_halo.insert(L->t_halo.end(), h.begin(), h.end());
      L->t_halo_ptr[t + 1] = (int)L->t_halo.size();
      L->max_halo = std::max(L->max_halo, (int)h.size());
    }
    {
      std::vector<char> in_halo(nC, 0);
      for (int dc : L->t_halo) in_halo[dc] = 1;
      L->n_halo_cells = 0;
      L->n_halo_cell_faces = 0;
      for (int dc = 0; dc < nC; ++dc)
        if (in_halo[dc]) {
          ++L->n_halo_cells;
          L->n_halo_cell_faces += L->c_ptr[dc + 1] - L->c_ptr[dc];
        }
    }
    if (kTileCells + L->max_halo >= 0xFFFF) {
      *err = "internal: tile halo too large for 16-bit local indices";
      return kEInval;
    }
    auto local = [&](int t, int dc) -> int {
      const int cb = t * kTileCells;
      if (dc >= cb && dc < cb + kTileCells) return dc - cb;
      const int* b = L->t_halo.data() + L->t_halo_ptr[t];
      const int* e = L->t_halo.data() + L->t_halo_ptr[t + 1];
      const int* p = std::lower_bound(b, e, dc);
      if (p == e || *p != dc) return -1;
      return kTileCells + (int)(p - b);
    };
    L->t_slot_loc.assign((size_t)nF + L->t_bor.size(), 0);
    for (int t = 0; t < nT; ++t) {
      const int ob = L->t_own_ptr[t], n_own = L->t_own_ptr[t + 1] - ob;
      const int bb = L->t_bor_ptr[t], n_bor = L->t_bor_ptr[t + 1] - bb;
      const size_t base = (size_t)ob + bb;
      for (int sl = 0; sl < n_own + n_bor; ++sl) {
        const int df = sl < n_own ? ob + sl : L->t_bor[bb + sl - n_own];
        const int l0 = local(t, L->f_c0c1[2 * (size_t)df]);
        const int c1 = L->f_c0c1[2 * (size_t)df + 1];
        const int l1 = c1 >= 0 ? local(t, c1) : 0xFFFF;
        if (l0 < 0 || l1 < 0) {
          *err = "internal: face cell missing from its tile table";
          return kEInval;
        }
        L->t_slot_loc[base + sl] = l0 | (l1 << 16);
      }
    }
    L->cf_nbl.assign(tot, 0);
    for (int dc = 0; dc < nC; ++dc) {
      const int t = tile_of(dc);
      for (int dk = L->c_ptr[dc]; dk < L->c_ptr[dc + 1]; ++dk) {
        const int nbm = L->cf_nb_fix[dk];
        const int nb = nbm & ((1 << kFvShift) - 1);
        const int l = local(t, nb);
        if (l < 0) {
          *err = "internal: neighbour missing from its tile table";
          return kEInval;
        }
        L->cf_nbl[dk] = l | ((nbm >> kFvShift) << 16);
      }
    }
  }
  return kOk;
}

int build_union(const std::vector<const HostMesh*>& parts, HostMesh* out,
                std::string* err) {
  HostMesh& u = *out;
  u = HostMesh{};
  if (parts.empty()) {
    *err = "empty batch";
    return kEInval;
  }
  const bool per = std::any_of(parts.begin(), parts.end(),
                               [](const HostMesh* p) { return p->periodic(); });
  u.case_cells.push_back(0);
  int zid = 1;
  for (size_t k = 0; k < parts.size(); ++k) {
    const HostMesh& p = *parts[k];
    if (!p.face_case.empty()) {
      *err = "a batch part is itself a batch";
      return kEInval;
    }
    const int on = u.n_nodes, oc = u.n_cells, of = u.n_faces;
    const int ot = (int)u.cell_faces.size();
    u.node_xy.insert(u.node_xy.end(), p.node_xy.begin(), p.node_xy.end());
    for (int v : p.face_nodes) u.face_nodes.push_back(v + on);
    for (size_t i = 0; i < p.face_cells.size(); ++i) {
      const int v = p.face_cells[i];
      u.face_cells.push_back(v >= 0 ? v + oc : -1);
    }
    u.face_type.insert(u.face_type.end(), p.face_type.begin(), p.face_type.end());
    if (per) {
      if (p.periodic()) u.c1_shift.insert(u.c1_shift.end(), p.c1_shift.begin(), p.c1_shift.end());
      else u.c1_shift.insert(u.c1_shift.end(), 2 * (size_t)p.n_faces, 0.0);
    }
    auto cat = [](auto& dst, const auto& src) { dst.insert(dst.end(), src.begin(), src.end()); };
    cat(u.face_ctr, p.face_ctr);
    cat(u.face_dir, p.face_dir);
    cat(u.face_area, p.face_area);
    cat(u.face_eta0, p.face_eta0);
    cat(u.face_dac, p.face_dac);
    cat(u.face_flag, p.face_flag);
    cat(u.face_flag_geo, p.face_flag_geo);
    if (u.cell_ptr.empty()) u.cell_ptr.push_back(0);
    for (int c = 0; c < p.n_cells; ++c) u.cell_ptr.push_back(p.cell_ptr[c + 1] + ot);
    for (int v : p.cell_faces) u.cell_faces.push_back(v + of);
    for (int v : p.cell_nb) u.cell_nb.push_back(v + oc);
    cat(u.cell_dof, p.cell_dof);
    cat(u.cell_eta0c, p.cell_eta0c);
    cat(u.cell_ctr, p.cell_ctr);
    cat(u.cell_vol, p.cell_vol);
    cat(u.cell_face_ctr, p.cell_face_ctr);
    for (int v : p.inner) u.inner.push_back(v + oc);
    for (int v : p.bond1) u.bond1.push_back(v + oc);
    for (int v : p.bond2) u.bond2.push_back(v + oc);
    for (int z = 0; z < p.n_zones(); ++z) {
      u.zone.push_back(zid++);
      u.zone.push_back(p.zone[4 * z + 1] + of);
      u.zone.push_back(p.zone[4 * z + 2] + of);
      u.zone.push_back(p.zone[4 * z + 3]);
    }
    u.face_case.insert(u.face_case.end(), p.n_faces, (int)k);
    u.n_nodes += p.n_nodes;
    u.n_cells += p.n_cells;
    u.n_faces += p.n_faces;
    u.case_cells.push_back(u.n_cells);
  }
  if ((long)parts.size() >= (1L << (31 - kInfoCaseShift))) {
    *err = "too many cases in one batch";
    return kEInval;
  }
  // every interior face is interpolated in the corrected face-value rule
  u.n_int_faces = u.n_faces;
  return kOk;
}


// ---------------------------------------------------------------------------
// 3D reader (MshBlock::splitInformationData3D / dataToMesh3D,
// mesh/MshBlock.cpp:436-789) and the reference's 3D geometry.
// ---------------------------------------------------------------------------
namespace {

typedef double V3[3];

inline void sub3(const double* a, const double* b, double* o) {
  o[0] = a[0] - b[0];
  o[1] = a[1] - b[1];
  o[2] = a[2] - b[2];
}
// Eigen-style dot / norm: left-to-right sums
inline double dot3(const double* a, const double* b) {
  double s = a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}
inline double norm3(const double* a) { return std::sqrt(dot3(a, a)); }

}  // namespace

int read_msh3d(const std::string& path, HostMesh3D* m, std::string* err) {
  std::ifstream in(path, std::ios::binary);
  if (!in) {
    *err = "cannot open " + path;
    return kEInval;
  }
  std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  std::vector<std::string> hdr, dat;
  dat.emplace_back();
  size_t b = 0;
  while (b < text.size()) {
    size_t e = text.find('\n', b);
    if (e == std::string::npos) e = text.size();
    std::string line = text.substr(b, e - b);
    while (!line.empty() && line.back() == '\r') line.pop_back();
    if (!line.empty() && (line[0] == '(' || line[0] == ')')) hdr.push_back(line);
    else dat.push_back(line);
    b = e + 1;
  }
  int nN = -1, nC = -1, nF = -1;
  for (const auto& s : hdr) {
    std::string br;
    if (s.size() < 3 || s[1] != '1' || !second_bracket(s, &br) || br.empty() || br[0] != '0')
      continue;
    auto t = split_spaces(br);
    if (t.size() < 3) continue;
    int v = hex_value(t[2]);
    if (s[2] == '0') nN = v;
    if (s[2] == '2') nC = v;
    if (s[2] == '3') nF = v;
  }
  if (nN <= 0 || nC <= 0 || nF <= 0) {
    *err = "missing node/cell/face totals";
    return kEMesh;
  }
  HostMesh3D& M = *m;
  M = HostMesh3D{};
  M.n_nodes = nN;
  M.n_cells = nC;
  M.n_faces = nF;
  M.node_xyz.assign(3 * (size_t)nN, 0.0);
  M.face_ptr.assign(1, 0);
  M.face_cells.assign(2 * (size_t)nF, -1);
  M.face_type.assign(nF, 0);
  size_t di = 0;
  int flag_node = 0, flag_face = 0;
  for (const auto& s : hdr) {
    std::string br;
    if (s.size() < 3 || s[1] != '1' || !second_bracket(s, &br) || br.empty() || br[0] == '0')
      continue;
    if (s[2] == '0') {
      ++di;  // the first data line is skipped, as in the 2D reader
      for (; flag_node < nN; ++flag_node) {
        if (di >= dat.size()) {
          *err = "node section truncated";
          return kEMesh;
        }
        auto t = split_spaces(dat[di++]);
        if (t.size() < 3) {
          *err = "bad 3D node line";
          return kEMesh;
        }
        for (int d = 0; d < 3; ++d)
          M.node_xyz[3 * (size_t)flag_node + d] = std::strtod(t[d].c_str(), nullptr);
      }
    } else if (s[2] == '3') {
      auto t = split_spaces(br);
      if (t.size() < 5) {
        *err = "bad face zone header";
        return kEMesh;
      }
      int zid = hex_value(t[0]), st = hex_value(t[1]), en = hex_value(t[2]), ty = hex_value(t[3]),
          nn = hex_value(t[4]);
      if (en > nF || st != flag_face + 1 || !(nn == 0 || nn == 3 || nn == 4)) {
        *err = "unsupported face zone (gaps or face node count other than 3, 4, mixed)";
        return kEMesh;
      }
      M.zone.insert(M.zone.end(), {zid, st, en, ty});
      if (ty == kInterior) M.n_int_faces = en;
      for (; flag_face < en; ++flag_face) {
        if (di >= dat.size()) {
          *err = "face section truncated";
          return kEMesh;
        }
        auto tk = split_spaces(dat[di++]);
        size_t p0 = 0;
        int k = nn;
        if (nn == 0) {  // mixed zone: the line starts with its node count
          if (tk.empty()) {
            *err = "bad mixed face line";
            return kEMesh;
          }
          k = hex_value(tk[0]);
          p0 = 1;
          if (k != 3 && k != 4) {
            *err = "mixed face with a node count other than 3 or 4";
            return kEMesh;
          }
        }
        const size_t need = p0 + k + ((ty == kInterior) ? 2 : 1);
        if (tk.size() < need) {
          *err = "bad face line";
          return kEMesh;
        }
        for (int j = 0; j < k; ++j) {
          const int nd = hex_value(tk[p0 + j]) - 1;
          if (nd < 0 || nd >= nN) {
            *err = "face references a missing node";
            return kEMesh;
          }
          M.face_nodes.push_back(nd);
        }
        M.face_ptr.push_back((int)M.face_nodes.size());
        const int c0 = hex_value(tk[p0 + k]) - 1;
        const int c1 = (ty == kInterior) ? hex_value(tk[p0 + k + 1]) - 1 : -1;
        if (c0 < 0 || c0 >= nC || (ty == kInterior && (c1 < 0 || c1 >= nC))) {
          *err = "face references a missing cell";
          return kEMesh;
        }
        M.face_cells[2 * (size_t)flag_face] = c0;
        M.face_cells[2 * (size_t)flag_face + 1] = c1;
        M.face_type[flag_face] = ty;
      }
    }
  }
  if (flag_node != nN || flag_face != nF || M.zone.empty()) {
    *err = "node or face sections incomplete";
    return kEMesh;
  }
  // cell -> face lists in file order (c0 then c1 of each face line), and
  // the neighbour per cell-face (the cell itself on boundary faces)
  std::vector<std::vector<int>> cf(nC), cn(nC);
  for (int f = 0; f < nF; ++f) {
    const int c0 = M.face_cells[2 * f], c1 = M.face_cells[2 * f + 1];
    cf[c0].push_back(f);
    if (c1 >= 0) {
      cf[c1].push_back(f);
      cn[c0].push_back(c1);
      cn[c1].push_back(c0);
    } else {
      cn[c0].push_back(c0);
    }
  }
  M.cell_ptr.assign(1, 0);
  for (int c = 0; c < nC; ++c) {
    if (cf[c].empty()) {
      *err = "cell without faces";
      return kEMesh;
    }
    M.cell_faces.insert(M.cell_faces.end(), cf[c].begin(), cf[c].end());
    M.cell_nb.insert(M.cell_nb.end(), cn[c].begin(), cn[c].end());
    M.cell_ptr.push_back((int)M.cell_faces.size());
  }
  // Face::setCenter (Face.cpp:8-39): centre = mean of nodes; area vector
  // 0.5 (n1-n0) x (n2-n0) for triangles, (n1-n0) x (n2-n0) for quads
  M.face_ctr.assign(3 * (size_t)nF, 0.0);
  M.face_dir.assign(3 * (size_t)nF, 0.0);
  M.face_area.assign(nF, 0.0);
  for (int f = 0; f < nF; ++f) {
    const int b0 = M.face_ptr[f], k = M.face_ptr[f + 1] - b0;
    double sm[3] = {0, 0, 0};
    for (int j = 0; j < k; ++j)
      for (int d = 0; d < 3; ++d) sm[d] += M.node_xyz[3 * (size_t)M.face_nodes[b0 + j] + d];
    for (int d = 0; d < 3; ++d) M.face_ctr[3 * (size_t)f + d] = sm[d] / (double)k;
    const double* p0 = &M.node_xyz[3 * (size_t)M.face_nodes[b0]];
    const double* p1 = &M.node_xyz[3 * (size_t)M.face_nodes[b0 + 1]];
    const double* p2 = &M.node_xyz[3 * (size_t)M.face_nodes[b0 + 2]];
    double f1[3], f2[3], cr[3];
    sub3(p1, p0, f1);
    sub3(p2, p0, f2);
    cr[0] = f1[1] * f2[2] - f1[2] * f2[1];
    cr[1] = f1[2] * f2[0] - f1[0] * f2[2];
    cr[2] = f1[0] * f2[1] - f1[1] * f2[0];
    double* dv = &M.face_dir[3 * (size_t)f];
    for (int d = 0; d < 3; ++d) dv[d] = (k == 3) ? 0.5 * cr[d] : cr[d];
    M.face_area[f] = norm3(dv);
  }
  // Cell::setCenter (mean of face centres) and setVolume (Cell.cpp:52-59,
  // the reference's 3D formula: sum of area (c - x_f) . n_f/|n_f| with the
  // stored face direction), and the corrected volume
  // V = 1/3 sum (x_f - c) . S_f(outward)
  M.cell_ctr.assign(3 * (size_t)nC, 0.0);
  M.cell_vol.assign(nC, 0.0);
  M.cell_vol_fixed.assign(nC, 0.0);
  for (int c = 0; c < nC; ++c) {
    double sm[3] = {0, 0, 0};
    const int kb = M.cell_ptr[c], ke = M.cell_ptr[c + 1];
    for (int k = kb; k < ke; ++k)
      for (int d = 0; d < 3; ++d) sm[d] += M.face_ctr[3 * (size_t)M.cell_faces[k] + d];
    double* cc = &M.cell_ctr[3 * (size_t)c];
    for (int d = 0; d < 3; ++d) cc[d] = sm[d] / (double)(ke - kb);
    double vol = 0, vfix = 0;
    for (int k = kb; k < ke; ++k) {
      const int f = M.cell_faces[k];
      const double* dv = &M.face_dir[3 * (size_t)f];
      const double nrm = norm3(dv);
      double u[3], tv[3];
      for (int d = 0; d < 3; ++d) u[d] = dv[d] / nrm;
      sub3(cc, &M.face_ctr[3 * (size_t)f], tv);
      double at[3];
      for (int d = 0; d < 3; ++d) at[d] = M.face_area[f] * tv[d];
      vol += dot3(at, u);
      // corrected: the face's area vector pointed out of this cell
      double xf[3];
      sub3(&M.face_ctr[3 * (size_t)f], cc, xf);
      double s = dot3(xf, dv);
      vfix += std::fabs(s);
    }
    M.cell_vol[c] = vol;
    M.cell_vol_fixed[c] = vfix / 3.0;
  }
  // orientation (MshBlock.cpp:632-648): where the area vector points into
  // c0 the face flips directAndCells and sets its left/right flags
  M.face_dac.assign(nF, 1);
  M.face_flag.assign(3 * (size_t)nF, 0);
  M.face_flag_set.assign(nF, 0);
  for (int f = 0; f < nF; ++f) {
    const double* dv = &M.face_dir[3 * (size_t)f];
    double t[3];
    sub3(&M.face_ctr[3 * (size_t)f], &M.cell_ctr[3 * (size_t)M.face_cells[2 * f]], t);
    if (dot3(dv, t) < 0) {
      M.face_dac[f] = -1;
      M.face_flag_set[f] = 1;
      for (int d = 0; d < 3; ++d) M.face_flag[3 * (size_t)f + d] = (-1 * dv[d] >= 0) ? 1 : 0;
    }
  }
  // directOfNbFaces, eta0, centre-middle difference, eta0C
  const int tot = M.cell_ptr[nC];
  M.cell_dof.assign(3 * (size_t)tot, 0.0);
  M.cell_eta0c.assign(tot, 0.0);
  M.face_eta0.assign(nF, 1.0);
  M.face_cmd.assign(3 * (size_t)nF, 0.0);
  for (int c = 0; c < nC; ++c)
    for (int k = M.cell_ptr[c]; k < M.cell_ptr[c + 1]; ++k) {
      const int f = M.cell_faces[k];
      const double s = (M.face_cells[2 * f] == c) ? M.face_dac[f] : -M.face_dac[f];
      for (int d = 0; d < 3; ++d) M.cell_dof[3 * (size_t)k + d] = s * M.face_dir[3 * (size_t)f + d];
    }
  for (int f = 0; f < nF; ++f) {
    const int c0 = M.face_cells[2 * f], c1 = M.face_cells[2 * f + 1];
    if (c1 >= 0) {
      double a[3], bb[3];
      sub3(&M.cell_ctr[3 * (size_t)c1], &M.face_ctr[3 * (size_t)f], a);
      sub3(&M.cell_ctr[3 * (size_t)c0], &M.face_ctr[3 * (size_t)f], bb);
      const double n1 = norm3(a);
      M.face_eta0[f] = n1 / (norm3(bb) + n1);
    }
  }
  for (int f = 0; f < M.n_int_faces && f < nF; ++f) {
    const int c0 = M.face_cells[2 * f], c1 = M.face_cells[2 * f + 1];
    if (c1 < 0) continue;
    for (int d = 0; d < 3; ++d) {
      const double mid = 0.5 * (M.cell_ctr[3 * (size_t)c0 + d] + M.cell_ctr[3 * (size_t)c1 + d]);
      M.face_cmd[3 * (size_t)f + d] = M.face_ctr[3 * (size_t)f + d] - mid;
    }
  }
  for (int c = 0; c < nC; ++c)
    for (int k = M.cell_ptr[c]; k < M.cell_ptr[c + 1]; ++k) {
      const int f = M.cell_faces[k];
      M.cell_eta0c[k] = (M.face_cells[2 * f] == c) ? M.face_eta0[f] : 1 - M.face_eta0[f];
    }
  // cell nodes (MshBlock.cpp:681-723): first appearance over the faces;
  // a 4-node cell is reordered by the angles at node 0
  M.cell_node_ptr.assign(1, 0);
  for (int c = 0; c < nC; ++c) {
    const size_t base = M.cell_nodes.size();
    for (int k = M.cell_ptr[c]; k < M.cell_ptr[c + 1]; ++k) {
      const int f = M.cell_faces[k];
      for (int j = M.face_ptr[f]; j < M.face_ptr[f + 1]; ++j) {
        const int nd = M.face_nodes[j];
        bool have = false;
        for (size_t i = base; i < M.cell_nodes.size(); ++i) have = have || M.cell_nodes[i] == nd;
        if (!have) M.cell_nodes.push_back(nd);
      }
    }
    if (M.cell_nodes.size() - base == 4) {
      int* p = &M.cell_nodes[base];
      double v1[3], v2[3], v3[3];
      sub3(&M.node_xyz[3 * (size_t)p[1]], &M.node_xyz[3 * (size_t)p[0]], v1);
      sub3(&M.node_xyz[3 * (size_t)p[2]], &M.node_xyz[3 * (size_t)p[0]], v2);
      sub3(&M.node_xyz[3 * (size_t)p[3]], &M.node_xyz[3 * (size_t)p[0]], v3);
      const double a12 = std::acos(dot3(v1, v2) / (norm3(v1) * norm3(v2)));
      const double a23 = std::acos(dot3(v3, v2) / (norm3(v3) * norm3(v2)));
      const double a13 = std::acos(dot3(v1, v3) / (norm3(v1) * norm3(v3)));
      if (a13 < a12 || a13 < a23) {
        if (a12 > a23) std::swap(p[2], p[3]);
        else std::swap(p[1], p[2]);
      }
    }
    M.cell_node_ptr.push_back((int)M.cell_nodes.size());
  }
  // boundary lists (as the 2D reader: MshBlock.cpp:727-743) and the count
  // of lower-id neighbours (:746-756)
  std::vector<uint8_t> bflag(nC, 0);
  for (int f = 0; f < nF; ++f)
    if (M.face_cells[2 * f + 1] < 0) {
      const int c0 = M.face_cells[2 * f];
      if (!bflag[c0]) {
        M.bond1.push_back(c0);
        bflag[c0] = 1;
      }
    }
  for (int c1 : M.bond1)
    for (int k = M.cell_ptr[c1]; k < M.cell_ptr[c1 + 1]; ++k) {
      const int nb = M.cell_nb[k];
      if (!bflag[nb]) {
        M.bond2.push_back(nb);
        bflag[nb] = 1;
      }
    }
  for (int c = 0; c < nC; ++c)
    if (!bflag[c]) M.inner.push_back(c);
  M.cell_nL.assign(nC, 0);
  for (int c = 0; c < nC; ++c)
    for (int k = M.cell_ptr[c]; k < M.cell_ptr[c + 1]; ++k) M.cell_nL[c] += (c > M.cell_nb[k]);
  return kOk;
}
}  // namespace mst
