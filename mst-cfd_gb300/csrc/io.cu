// Result writer and checkpoint files of the density-based path.
//
//   mst_node_values / mst_write_plt
//       Work::writedataRhoBasedMshNodePlt (work/Work.cpp:204-319): face values
//       (eta0 blend on interior faces, the cell value on boundary faces),
//       averaged onto the nodes with 1/area weights, then the Tecplot ASCII
//       POINT zone X Y rho u v T p Ma and the element connectivity.  The
//       averaging runs on the device (k_node_average, one thread per node);
//       the host only formats the text, in parallel chunks.
//   mst_write_cell_text / mst_read_cell_text
//       the text checkpoint of Work::writedataCellContinue (Work.cpp:483-514)
//       and its reader Work::readPbasedCellPlt (Work.cpp:432-482).
//   mst_checkpoint_save / mst_checkpoint_load
//       an exact binary checkpoint (state, float-pair parts on the FP32 path,
//       time), tied to its mesh by a hash and guarded by a checksum.
//
// This file is compiled without FMA contraction: the node averages round
// every operation in the reference's order, so a reference-mode .plt is
// byte-identical to the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "ctx.hpp"
#include "physics.cuh"

namespace {

#define IO_CU(call)                                                            \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return mst_internal_fail(MST_ECUDA, std::string(#call) + ": " +          \
                                              cudaGetErrorString(e_));         \
  } while (0)

// ---------------------------------------------------------------------------
// device: node averaging
// ---------------------------------------------------------------------------
// One thread per node (file node order).  Entry e of node i is one face the
// node lies on, in ascending face id (the order MshBlock.cpp:231-232 builds
// Node::pNbFaces): the face's two device cells (c1 < 0: boundary face, the
// face value is the c0 cell value) and (eta0, weight).
template <bool PAIRS>
__global__ void k_node_average(int n_nodes, const int* __restrict__ ptr,
                               const int2* __restrict__ cells,
                               const double2* __restrict__ ew,
                               const double4_32a* __restrict__ q,
                               const float4* __restrict__ qh,
                               const float4* __restrict__ ql, double cv,
                               double* __restrict__ node_q,
                               double* __restrict__ node_vars) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  double d = 0.0;
  for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
    const int2 c = cells[e];
    const double2 x = ew[e];
    double q0[4], fq[4];
    if (PAIRS) {
      const float4 h = qh[c.x], l = ql[c.x];
      q0[0] = (double)h.x + (double)l.x;
      q0[1] = (double)h.y + (double)l.y;
      q0[2] = (double)h.z + (double)l.z;
      q0[3] = (double)h.w + (double)l.w;
    } else {
      const double4_32a v = q[c.x];
      q0[0] = v.x; q0[1] = v.y; q0[2] = v.z; q0[3] = v.w;
    }
    if (c.y >= 0) {
      double q1[4];
      if (PAIRS) {
        const float4 h = qh[c.y], l = ql[c.y];
        q1[0] = (double)h.x + (double)l.x;
        q1[1] = (double)h.y + (double)l.y;
        q1[2] = (double)h.z + (double)l.z;
        q1[3] = (double)h.w + (double)l.w;
      } else {
        const double4_32a v = q[c.y];
        q1[0] = v.x; q1[1] = v.y; q1[2] = v.z; q1[3] = v.w;
      }
      // pFaceQ = eta0 Q0; pFaceQ += (1 - eta0) Q1  (Work.cpp:250-251)
      const double om = 1.0 - x.x;
#pragma unroll
      for (int j = 0; j < 4; ++j) fq[j] = x.x * q0[j] + om * q1[j];
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) fq[j] = q0[j];
    }
    // pNodeQ += w * pFaceQ; d += w  (Work.cpp:291-294)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] += x.y * fq[j];
    d += x.y;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) acc[j] /= d;
  if (node_q) {
#pragma unroll
    for (int j = 0; j < 4; ++j) node_q[4 * (size_t)i + j] = acc[j];
  }
  if (node_vars) {
    // getT / getP / getMa (work/FUNCTION.cpp:8-20), in their evaluation order
    const double rho = acc[0], m1 = acc[1], m2 = acc[2], E = acc[3];
    const double ke = 0.5 * (m1 * m1 + m2 * m2) / rho;
    const double T = (E - ke) / rho / cv;
    const double p = (E - ke) * mst::Gas<double>::gm1();
    const double ma = sqrt((m1 * m1 + m2 * m2) / (mst::Gas<double>::gamma() * p * rho));
    double* o = node_vars + 6 * (size_t)i;
    o[0] = rho;
    o[1] = m1 / rho;
    o[2] = m2 / rho;
    o[3] = T;
    o[4] = p;
    o[5] = ma;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host: node -> face entries (built once per context and weighting rule)
// ---------------------------------------------------------------------------
struct mst_node_avg {
  int quirks = -1;
  int n_nodes = 0;
  int* ptr = nullptr;
  int2* cells = nullptr;
  double2* ew = nullptr;
  double* out_q = nullptr;
  double* out_vars = nullptr;
};

// Frees the writer's buffers of a context (called by mst_ctx_destroy).
void mst_io_release(mst_ctx* c) {
  mst_node_avg* a = c->node_avg;
  if (!a) return;
  cudaFree(a->ptr);
  cudaFree(a->cells);
  cudaFree(a->ew);
  cudaFree(a->out_q);
  cudaFree(a->out_vars);
  delete a;
  c->node_avg = nullptr;
}

namespace {

typedef mst_node_avg NodeAvg;

// Reference face types handled by the writer's face-value switch
// (Work.cpp:244-283): 2 interior (eta0 blend), 10 inlet, 3 wall, 5 outlet
// (cell value).  Other types (symmetry 7 ...) are left unset there; here
// they take the cell value too.
mst_status build_node_avg(mst_ctx* c, int quirks, NodeAvg* a) {
  const mst::HostMesh& m = c->mesh->host;
  const mst::DevLayout& L = c->mesh->lay;
  const int nN = m.n_nodes, nF = m.n_faces;
  if (quirks && nN > nF)
    return mst_internal_fail(MST_EINVAL,
                             "reference node weighting reads face areas by node id; the mesh "
                             "has more nodes than faces");
  std::vector<int> ptr(nN + 1, 0);
  for (int f = 0; f < nF; ++f)
    for (int k = 0; k < 2; ++k) ptr[m.face_nodes[2 * f + k] + 1]++;
  for (int i = 0; i < nN; ++i) ptr[i + 1] += ptr[i];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  std::vector<int2> cells(ptr[nN]);
  std::vector<double2> ew(ptr[nN]);
  for (int f = 0; f < nF; ++f) {
    const int c0 = L.cell_perm[m.face_cells[2 * f]];
    const bool interior = m.face_type[f] == mst::kInterior;
    const int c1 = interior ? L.cell_perm[m.face_cells[2 * f + 1]] : -1;
    for (int k = 0; k < 2; ++k) {
      const int n = m.face_nodes[2 * f + k];
      const int e = fill[n]++;
      cells[e] = make_int2(c0, c1);
      // the reference weights every face of node n by 1 / area[n]
      // (Work.cpp:292-293 index the face list by the node id); the fixed
      // rule weights each face by its own 1 / area
      const double w = quirks ? 1 / m.face_area[n] : 1 / m.face_area[f];
      ew[e] = make_double2(interior ? m.face_eta0[f] : 1.0, w);
    }
  }
  cudaFree(a->ptr);
  cudaFree(a->cells);
  cudaFree(a->ew);
  cudaFree(a->out_q);
  cudaFree(a->out_vars);
  *a = NodeAvg{};
  IO_CU(cudaMalloc(&a->ptr, sizeof(int) * ptr.size()));
  IO_CU(cudaMalloc(&a->cells, sizeof(int2) * std::max<size_t>(cells.size(), 1)));
  IO_CU(cudaMalloc(&a->ew, sizeof(double2) * std::max<size_t>(ew.size(), 1)));
  IO_CU(cudaMalloc(&a->out_q, sizeof(double) * 4 * std::max(nN, 1)));
  IO_CU(cudaMalloc(&a->out_vars, sizeof(double) * 6 * std::max(nN, 1)));
  IO_CU(cudaMemcpy(a->ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice));
  if (!cells.empty()) {
    IO_CU(cudaMemcpy(a->cells, cells.data(), sizeof(int2) * cells.size(),
                     cudaMemcpyHostToDevice));
    IO_CU(cudaMemcpy(a->ew, ew.data(), sizeof(double2) * ew.size(), cudaMemcpyHostToDevice));
  }
  a->quirks = quirks;
  a->n_nodes = nN;
  return MST_OK;
}

// Runs the node averaging of the current state; results in a->out_q/out_vars.
mst_status node_average(mst_ctx* c, NodeAvg** out) {
  if (!c->node_avg) c->node_avg = new NodeAvg();
  NodeAvg* a = c->node_avg;
  const int quirks = c->p.reference_quirks ? 1 : 0;
  if (a->quirks != quirks) {
    mst_status s = build_node_avg(c, quirks, a);
    if (s) return s;
  }
  const int nN = a->n_nodes;
  if (nN > 0) {
    const int nb = (nN + 127) / 128;
    if (c->p.precision == MST_PREC_FP32)
      k_node_average<true><<<nb, 128, 0, c->stream>>>(nN, a->ptr, a->cells, a->ew, nullptr,
                                                       c->qf_old, c->ql_old, c->p.cv,
                                                       a->out_q, a->out_vars);
    else
      k_node_average<false><<<nb, 128, 0, c->stream>>>(nN, a->ptr, a->cells, a->ew, c->q_old,
                                                        nullptr, nullptr, c->p.cv, a->out_q,
                                                        a->out_vars);
    IO_CU(cudaGetLastError());
  }
  *out = a;
  return MST_OK;
}

// ---------------------------------------------------------------------------
// host: cell -> node connectivity in the reference's order
// ---------------------------------------------------------------------------
// MshBlock.cpp:335-367: for each face of the cell (ascending face id), each
// of its nodes not yet listed is appended; in a 4-node cell, nodes 2 and 3
// swap when the dot product of n0 - n1 and n2 - n3 is negative.
void cell_nodes(const mst::HostMesh& m, std::vector<int>& ptr, std::vector<int>& ids) {
  const int nC = m.n_cells;
  ptr.assign(nC + 1, 0);
  ids.clear();
  ids.reserve((size_t)nC * 4);
  for (int c = 0; c < nC; ++c) {
    const size_t base = ids.size();
    for (int k = m.cell_ptr[c]; k < m.cell_ptr[c + 1]; ++k) {
      const int f = m.cell_faces[k];
      for (int j = 0; j < 2; ++j) {
        const int n = m.face_nodes[2 * f + j];
        bool have = false;
        for (size_t i = base; i < ids.size(); ++i) have = have || ids[i] == n;
        if (!have) ids.push_back(n);
      }
    }
    if (ids.size() - base == 4) {
      const double* p0 = &m.node_xy[2 * (size_t)ids[base]];
      const double* p1 = &m.node_xy[2 * (size_t)ids[base + 1]];
      const double* p2 = &m.node_xy[2 * (size_t)ids[base + 2]];
      const double* p3 = &m.node_xy[2 * (size_t)ids[base + 3]];
      double dot = (p0[0] - p1[0]) * (p2[0] - p3[0]);
      dot += (p0[1] - p1[1]) * (p2[1] - p3[1]);
      if (dot < 0) std::swap(ids[base + 2], ids[base + 3]);
    }
    ptr[c + 1] = (int)ids.size();
  }
}

// ---------------------------------------------------------------------------
// host: text formatting ("%.15f": fixed, 15 decimals, as the reference's
// `fixed << setprecision(15)` streams; the setw(15) it also sets never pads,
// since every such number is at least 17 characters long)
// ---------------------------------------------------------------------------
inline void put_fixed(std::string& s, double v) {
  char buf[400];
  auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::fixed, 15);
  s.append(buf, r.ptr);
}

inline void put_int(std::string& s, long v) {
  char buf[24];
  auto r = std::to_chars(buf, buf + sizeof buf, v);
  s.append(buf, r.ptr);
}

// Formats rows [0, n) with fn(i, string&) on all host threads, in order.
template <class F>
std::vector<std::string> format_parallel(size_t n, F fn) {
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = (unsigned)std::min<size_t>(nt, std::max<size_t>(1, n / 4096));
  std::vector<std::string> parts(nt);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) {
    th.emplace_back([&, t] {
      const size_t b = n * t / nt, e = n * (t + 1) / nt;
      std::string& s = parts[t];
      s.reserve((e - b) * 80);
      for (size_t i = b; i < e; ++i) fn(i, s);
    });
  }
  for (auto& x : th) x.join();
  return parts;
}

bool write_all(FILE* f, const std::string& s) {
  return s.empty() || std::fwrite(s.data(), 1, s.size(), f) == s.size();
}

// FNV-1a, 64 bit, over bytes
uint64_t fnv1a(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t mesh_hash(const mst::HostMesh& m) {
  uint64_t h = fnv1a(&m.n_nodes, sizeof(int));
  h = fnv1a(&m.n_cells, sizeof(int), h);
  h = fnv1a(&m.n_faces, sizeof(int), h);
  h = fnv1a(m.node_xy.data(), m.node_xy.size() * sizeof(double), h);
  h = fnv1a(m.face_nodes.data(), m.face_nodes.size() * sizeof(int), h);
  h = fnv1a(m.face_cells.data(), m.face_cells.size() * sizeof(int), h);
  h = fnv1a(m.face_type.data(), m.face_type.size() * sizeof(int), h);
  return h;
}

struct CkptHeader {
  char magic[8];          // "MSTCKPT" + NUL
  uint32_t version;       // 1
  uint32_t header_bytes;  // sizeof(CkptHeader)
  uint64_t n_cells;
  uint64_t mesh_hash;
  uint32_t n_vars;        // 4
  uint32_t precision;     // MST_PREC_* of the writing context
  uint32_t has_pairs;     // float-pair parts follow the FP64 state
  uint32_t reserved;
  double time;
  double dt;              // last step length
  uint64_t payload_bytes;
  uint64_t payload_hash;  // FNV-1a 64 of the payload
  uint64_t header_hash;   // FNV-1a 64 of the header up to this field
};
static_assert(sizeof(CkptHeader) == 88, "checkpoint header layout");

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

mst_status mst_node_values(mst_ctx* c, double* node_q, double* node_vars) {
  if (!c) return mst_internal_fail(MST_EINVAL, "NULL context");
  NodeAvg* a = nullptr;
  mst_status s = node_average(c, &a);
  if (s) return s;
  const int nN = a->n_nodes;
  if (node_q && nN)
    IO_CU(cudaMemcpyAsync(node_q, a->out_q, sizeof(double) * 4 * nN, cudaMemcpyDeviceToHost,
                          c->stream));
  if (node_vars && nN)
    IO_CU(cudaMemcpyAsync(node_vars, a->out_vars, sizeof(double) * 6 * nN,
                          cudaMemcpyDeviceToHost, c->stream));
  IO_CU(cudaStreamSynchronize(c->stream));
  return MST_OK;
}

mst_status mst_write_plt(mst_ctx* c, const char* path, int zone_t) {
  if (!c || !path) return mst_internal_fail(MST_EINVAL, "NULL argument");
  const mst::HostMesh& m = c->mesh->host;
  const int nN = m.n_nodes, nC = m.n_cells;
  const bool ref = c->p.reference_quirks != 0;
  std::vector<double> vars((size_t)nN * 6);
  mst_status s = mst_node_values(c, nullptr, vars.data());
  if (s) return s;
  std::vector<int> cptr, cids;
  cell_nodes(m, cptr, cids);
  bool all_tri = true, all_le4 = true;
  for (int i = 0; i < nC; ++i) {
    const int k = cptr[i + 1] - cptr[i];
    all_tri = all_tri && k == 3;
    all_le4 = all_le4 && k <= 4;
  }
  if (!ref && !all_le4)
    return mst_internal_fail(MST_EINVAL, "cells with more than 4 nodes have no Tecplot zone type");
  FILE* f = std::fopen(path, "wb");
  if (!f) return mst_internal_fail(MST_EINVAL, std::string("cannot write ") + path);
  std::string head;
  // Work.cpp:223-237; the reference's title line opens with a stray quote
  // and its zone type is the compile-time FELNUM 4 (CONST.h:5)
  head += ref ? "\"TITLE = \"Example: Variable and Connectivity List Sharing\"\n"
              : "TITLE = \"Example: Variable and Connectivity List Sharing\"\n";
  head += "VARIABLES = \"X\", \"Y\", \"rho\" , \"u\" , \"v\" , \"T\" , \"p\" , \"Ma\" \n";
  head += "ZONE T=\"";
  put_int(head, zone_t);
  head += "\", DATAPACKING=POINT, NODES=";
  put_int(head, nN);
  head += ", ELEMENTS=";
  put_int(head, nC);
  head += (!ref && all_tri) ? ", ZONETYPE=FETRIANGLE\n" : ", ZONETYPE=FEQUADRILATERAL\n";
  bool ok = write_all(f, head);
  // node rows: X Y rho u v T p Ma, each followed by a space (Work.cpp:296-303)
  auto rows = format_parallel((size_t)nN, [&](size_t i, std::string& t) {
    put_fixed(t, m.node_xy[2 * i]);
    t += ' ';
    put_fixed(t, m.node_xy[2 * i + 1]);
    t += ' ';
    const double* v = &vars[6 * i];
    for (int k = 0; k < 6; ++k) {
      put_fixed(t, v[k]);
      t += ' ';
    }
    t += '\n';
  });
  for (auto& p : rows) ok = ok && write_all(f, p);
  // connectivity: 1-based node ids, each followed by a space (Work.cpp:305-311).
  // The reader's order makes n0 - n1 and n2 - n3 point the same way, so a
  // quad written 0 1 2 3 (as the reference does) is a bow tie; the cyclic
  // order is 0 1 3 2 (the order of Work.cpp:412-415).  A valid
  // FEQUADRILATERAL zone also repeats a triangle's last node.
  auto conn = format_parallel((size_t)nC, [&](size_t i, std::string& t) {
    const int b = cptr[i], e = cptr[i + 1];
    static const int cyc[4] = {0, 1, 3, 2};
    for (int k = b; k < e; ++k) {
      const int kk = (!ref && e - b == 4) ? b + cyc[k - b] : k;
      put_int(t, cids[kk] + 1);
      t += ' ';
    }
    if (!ref && !all_tri && e - b == 3) {
      put_int(t, cids[e - 1] + 1);
      t += ' ';
    }
    t += '\n';
  });
  for (auto& p : conn) ok = ok && write_all(f, p);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return mst_internal_fail(MST_EINVAL, std::string("write failed: ") + path);
  return MST_OK;
}

mst_status mst_write_cell_text(mst_ctx* c, const char* path) {
  if (!c || !path) return mst_internal_fail(MST_EINVAL, "NULL argument");
  const int nC = c->mesh->host.n_cells;
  std::vector<double> q((size_t)nC * 4);
  mst_status s = mst_get_state(c, q.data(), 4);
  if (s) return s;
  FILE* f = std::fopen(path, "wb");
  if (!f) return mst_internal_fail(MST_EINVAL, std::string("cannot write ") + path);
  auto rows = format_parallel((size_t)nC, [&](size_t i, std::string& t) {
    for (int k = 0; k < 4; ++k) {
      put_fixed(t, q[4 * i + k]);
      t += ' ';
    }
    t += '\n';
  });
  bool ok = true;
  for (auto& p : rows) ok = ok && write_all(f, p);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return mst_internal_fail(MST_EINVAL, std::string("write failed: ") + path);
  return MST_OK;
}

mst_status mst_read_cell_text(mst_ctx* c, const char* path) {
  if (!c || !path) return mst_internal_fail(MST_EINVAL, "NULL argument");
  const int nC = c->mesh->host.n_cells;
  FILE* f = std::fopen(path, "rb");
  if (!f) return mst_internal_fail(MST_EINVAL, std::string("cannot open ") + path);
  std::string text;
  {
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    std::fclose(f);
  }
  std::vector<double> q((size_t)nC * 4);
  size_t pos = 0;
  for (int i = 0; i < nC; ++i) {
    const size_t eol = std::min(text.find('\n', pos), text.size());
    if (pos >= text.size())
      return mst_internal_fail(MST_EINVAL, std::string(path) + ": " + std::to_string(i) +
                                               " lines, the mesh has " + std::to_string(nC) +
                                               " cells");
    // one line: the first 4 space-separated numbers (Work.cpp:463-474)
    size_t p = pos;
    for (int k = 0; k < 4; ++k) {
      const size_t sp = std::min(text.find(' ', p), eol);
      std::string tok = text.substr(p, sp - p);
      while (!tok.empty() && (tok.back() == '\r')) tok.pop_back();
      char* end = nullptr;
      const double v = std::strtod(tok.c_str(), &end);
      if (tok.empty() || end == tok.c_str())
        return mst_internal_fail(MST_EINVAL, std::string(path) + ": line " +
                                                 std::to_string(i + 1) + " has fewer than 4 numbers");
      q[4 * (size_t)i + k] = v;
      p = std::min(sp + 1, eol);
    }
    pos = eol + 1;
  }
  return mst_set_state(c, q.data(), 4);
}

mst_status mst_checkpoint_save(mst_ctx* c, const char* path) {
  if (!c || !path) return mst_internal_fail(MST_EINVAL, "NULL argument");
  const mst::HostMesh& m = c->mesh->host;
  const int nC = m.n_cells;
  const bool pairs = c->p.precision == MST_PREC_FP32;
  std::vector<double> q((size_t)nC * 4);
  mst_status s = mst_get_state(c, q.data(), 4);
  if (s) return s;
  std::vector<float> hl;
  if (pairs) {
    // hi and lo parts in file cell order: device rows gathered on the host
    std::vector<float> hi((size_t)nC * 4), lo((size_t)nC * 4);
    IO_CU(cudaMemcpyAsync(hi.data(), c->qf_old, sizeof(float) * 4 * nC, cudaMemcpyDeviceToHost,
                          c->stream));
    IO_CU(cudaMemcpyAsync(lo.data(), c->ql_old, sizeof(float) * 4 * nC, cudaMemcpyDeviceToHost,
                          c->stream));
    IO_CU(cudaStreamSynchronize(c->stream));
    hl.resize((size_t)nC * 8);
    const std::vector<int>& perm = c->mesh->lay.cell_perm;
    for (int i = 0; i < nC; ++i)
      for (int k = 0; k < 4; ++k) {
        hl[4 * (size_t)i + k] = hi[4 * (size_t)perm[i] + k];
        hl[4 * ((size_t)nC + i) + k] = lo[4 * (size_t)perm[i] + k];
      }
  }
  double sc[4];
  IO_CU(cudaMemcpyAsync(sc, c->scal, sizeof sc, cudaMemcpyDeviceToHost, c->stream));
  IO_CU(cudaStreamSynchronize(c->stream));
  CkptHeader h{};
  std::memcpy(h.magic, "MSTCKPT", 8);
  h.version = 1;
  h.header_bytes = sizeof(CkptHeader);
  h.n_cells = (uint64_t)nC;
  h.mesh_hash = mesh_hash(m);
  h.n_vars = 4;
  h.precision = (uint32_t)c->p.precision;
  h.has_pairs = pairs ? 1 : 0;
  h.time = sc[1];
  h.dt = sc[0];
  h.payload_bytes = q.size() * sizeof(double) + hl.size() * sizeof(float);
  uint64_t ph = fnv1a(q.data(), q.size() * sizeof(double));
  if (!hl.empty()) ph = fnv1a(hl.data(), hl.size() * sizeof(float), ph);
  h.payload_hash = ph;
  h.header_hash = fnv1a(&h, offsetof(CkptHeader, header_hash));
  FILE* f = std::fopen(path, "wb");
  if (!f) return mst_internal_fail(MST_EINVAL, std::string("cannot write ") + path);
  bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
  ok = ok && std::fwrite(q.data(), sizeof(double), q.size(), f) == q.size();
  if (!hl.empty()) ok = ok && std::fwrite(hl.data(), sizeof(float), hl.size(), f) == hl.size();
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return mst_internal_fail(MST_EINVAL, std::string("write failed: ") + path);
  return MST_OK;
}

mst_status mst_checkpoint_load(mst_ctx* c, const char* path) {
  if (!c || !path) return mst_internal_fail(MST_EINVAL, "NULL argument");
  const mst::HostMesh& m = c->mesh->host;
  const int nC = m.n_cells;
  FILE* f = std::fopen(path, "rb");
  if (!f) return mst_internal_fail(MST_EINVAL, std::string("cannot open ") + path);
  CkptHeader h{};
  const bool got = std::fread(&h, sizeof h, 1, f) == 1;
  auto bad = [&](const std::string& why) {
    std::fclose(f);
    return mst_internal_fail(MST_EINVAL, std::string(path) + ": " + why);
  };
  if (!got || std::memcmp(h.magic, "MSTCKPT", 8) != 0) return bad("not a checkpoint");
  if (h.version != 1 || h.header_bytes != sizeof(CkptHeader))
    return bad("unsupported checkpoint version");
  if (h.header_hash != fnv1a(&h, offsetof(CkptHeader, header_hash)))
    return bad("header checksum mismatch");
  if (h.n_cells != (uint64_t)nC || h.n_vars != 4) return bad("cell count differs from the mesh");
  if (h.mesh_hash != mesh_hash(m)) return bad("written for another mesh");
  const size_t nq = (size_t)nC * 4, nhl = h.has_pairs ? (size_t)nC * 8 : 0;
  if (h.payload_bytes != nq * sizeof(double) + nhl * sizeof(float))
    return bad("payload size mismatch");
  std::vector<double> q(nq);
  std::vector<float> hl(nhl);
  bool ok = std::fread(q.data(), sizeof(double), nq, f) == nq;
  if (nhl) ok = ok && std::fread(hl.data(), sizeof(float), nhl, f) == nhl;
  std::fclose(f);
  if (!ok) return mst_internal_fail(MST_EINVAL, std::string(path) + ": truncated");
  uint64_t ph = fnv1a(q.data(), nq * sizeof(double));
  if (nhl) ph = fnv1a(hl.data(), nhl * sizeof(float), ph);
  if (ph != h.payload_hash)
    return mst_internal_fail(MST_EINVAL, std::string(path) + ": payload checksum mismatch");
  mst_status s = mst_set_state(c, q.data(), 4);
  if (s) return s;
  if (nhl && c->p.precision == MST_PREC_FP32) {
    // the exact float pairs (hi + lo in double may round), device order
    const std::vector<int>& perm = c->mesh->lay.cell_perm;
    std::vector<float> hi(nq), lo(nq);
    for (int i = 0; i < nC; ++i)
      for (int k = 0; k < 4; ++k) {
        hi[4 * (size_t)perm[i] + k] = hl[4 * (size_t)i + k];
        lo[4 * (size_t)perm[i] + k] = hl[4 * ((size_t)nC + i) + k];
      }
    IO_CU(cudaMemcpyAsync(c->qf_old, hi.data(), sizeof(float) * nq, cudaMemcpyHostToDevice,
                          c->stream));
    IO_CU(cudaMemcpyAsync(c->ql_old, lo.data(), sizeof(float) * nq, cudaMemcpyHostToDevice,
                          c->stream));
    IO_CU(cudaMemcpyAsync(c->qf_new, c->qf_old, sizeof(float) * nq, cudaMemcpyDeviceToDevice,
                          c->stream));
    IO_CU(cudaMemcpyAsync(c->ql_new, c->ql_old, sizeof(float) * nq, cudaMemcpyDeviceToDevice,
                          c->stream));
  }
  double sc[4];
  IO_CU(cudaMemcpyAsync(sc, c->scal, sizeof sc, cudaMemcpyDeviceToHost, c->stream));
  IO_CU(cudaStreamSynchronize(c->stream));
  sc[0] = h.dt;
  sc[1] = h.time;
  IO_CU(cudaMemcpyAsync(c->scal, sc, 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  IO_CU(cudaStreamSynchronize(c->stream));
  return MST_OK;
}

}  // extern "C"
