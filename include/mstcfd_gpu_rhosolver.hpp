// Drop-in replacement for MST-CFD's RhoSolver (rhoSolver/RhoSolver.h:14-56)
// that runs solve() on the GB300 through the C ABI of mstcfd.h.
//
// Same public surface as the reference class:
//   GpuRhoSolver(MshBlock*, fstream*, AllData*); setDT(NUM); solve();
//   getOldValue(); getOldNTimeValue(); getNewValue(); updateNewToOld();
// so Time::goNextTimeStep (time/Time.cpp:57-61) can construct it in place of
// RhoSolver.  The reference constructs its solver every time step
// (Time.cpp:58), so the mesh upload is cached per MshBlock pointer: the
// first construction for a mesh uploads it, later ones reuse it.
//
// solve() copies AllData's old state (p1OldCellQs, an array of Eigen
// Matrix<double,4,1>) to the GPU, runs the residual and the explicit update,
// and writes p1NewCellQs back, bit-identical to the reference in the default
// arithmetic (MST_PREC_FP64_EXACT with the reference's quirks).  The flux
// scheme and order follow the reference's CONST.h macros when they are
// visible (RHOSOLVER, ACCURACY); set_params() overrides them.
//
// Errors: the reference has no error path; this class writes the message to
// the solver's log stream (when given) and throws std::runtime_error.
#pragma once
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "mstcfd.h"

namespace mstcfd {

namespace detail {
struct MeshEntry {
  mst_mesh* mesh = nullptr;
  mst_ctx* ctx = nullptr;
  int n_cells = 0;
};
inline std::map<const void*, MeshEntry>& mesh_cache() {
  static std::map<const void*, MeshEntry> m;
  return m;
}
inline mst_params& default_params() {
  static mst_params p = [] {
    mst_params q;
    mst_params_default(&q);
    return q;
  }();
  return p;
}
}  // namespace detail

// Parameters used by every GpuRhoSolver created afterwards.
inline void set_params(const mst_params& p) { detail::default_params() = p; }

// Releases the cached device copy of a mesh (e.g. before freeing it).
inline void release_mesh(const void* msh_block) {
  auto& c = detail::mesh_cache();
  auto it = c.find(msh_block);
  if (it == c.end()) return;
  mst_ctx_destroy(it->second.ctx);
  mst_mesh_destroy(it->second.mesh);
  c.erase(it);
}

template <class MshBlockT, class AllDataT, class VecT>
class GpuRhoSolverT {
 public:
  GpuRhoSolverT(MshBlockT* mesh, std::fstream* log, AllDataT* data)
      : mesh_(mesh), log_(log), data_(data), dt_(1.0 / 4e+3) {
    static_assert(sizeof(VecT) % sizeof(double) == 0, "state rows of doubles");
    auto& cache = detail::mesh_cache();
    auto it = cache.find(mesh);
    if (it == cache.end()) it = cache.emplace(mesh, upload(mesh)).first;
    entry_ = &it->second;
  }

  void setDT(double dt) { dt_ = dt; }

  void solve() {
    const size_t stride = sizeof(VecT) / sizeof(double);
    check(mst_set_dt(entry_->ctx, dt_));
    check(mst_set_state(entry_->ctx, first(data_->getP1OldCellQs()), stride));
    check(mst_solve(entry_->ctx));
    check(mst_get_new_state(entry_->ctx, first(data_->getP1NewCellQs()), stride));
  }

  VecT* getOldValue() { return data_->getP1OldCellQs(); }
  VecT* getOldNTimeValue() { return data_->getPtP1OldNTimeCellQs(); }
  VecT* getNewValue() { return data_->getP1NewCellQs(); }

  // host copy new -> old, as the reference does (RhoSolver.cpp:513-517)
  void updateNewToOld() {
    VecT* o = data_->getP1OldCellQs();
    VecT* n = data_->getP1NewCellQs();
    for (int i = 0; i < entry_->n_cells; ++i) o[i] = n[i];
  }

 private:
  static double* first(VecT* v) { return reinterpret_cast<double*>(&v[0]); }

  void check(mst_status s) {
    if (s == MST_OK) return;
    std::string msg = std::string("GpuRhoSolver: ") + mst_last_error();
    if (log_ && log_->is_open()) (*log_) << msg << std::endl;
    throw std::runtime_error(msg);
  }

  // MshBlock -> mst_mesh_desc through the reference's public getters
  // (mesh/MshBlock.h:19-45, Face.h:10-41, Node.h, FacesInf.h)
  detail::MeshEntry upload(MshBlockT* m) {
    const int nN = m->getNumOfNodes(), nC = m->getNumOfCells(),
              nF = m->getNumOfFaces(), nZ = m->getNumOfFacesInfs();
    std::vector<double> xy(2 * (size_t)nN);
    auto nodes = m->getBeginItNodesList();
    for (int i = 0; i < nN; ++i) {
      xy[2 * i] = nodes[i].getCenter()(0);
      xy[2 * i + 1] = nodes[i].getCenter()(1);
    }
    std::vector<int> fn(2 * (size_t)nF), fc(2 * (size_t)nF);
    auto faces = m->getBeginItFacesList();
    for (int i = 0; i < nF; ++i) {
      auto nb = faces[i].getBeginItPNbNodes();
      fn[2 * i] = nb[0]->getId();
      fn[2 * i + 1] = nb[1]->getId();
      auto cb = faces[i].getBeginItPNbCells();
      fc[2 * i] = cb[0]->getId();
      fc[2 * i + 1] = faces[i].getNumOfpNbCells() > 1 ? cb[1]->getId() : -1;
    }
    std::vector<int> zones(4 * (size_t)nZ);
    auto zi = m->getBeginItFacesInfList();
    for (int z = 0; z < nZ; ++z) {
      zones[4 * z] = zi[z].getNumber();
      zones[4 * z + 1] = zi[z].getStart();
      zones[4 * z + 2] = zi[z].getEnd();
      zones[4 * z + 3] = zi[z].getType();
    }
    mst_mesh_desc d{};
    d.n_nodes = nN;
    d.node_xy = xy.data();
    d.n_cells = nC;
    d.n_faces = nF;
    d.face_nodes = fn.data();
    d.face_cells = fc.data();
    d.n_zones = nZ;
    d.zones = zones.data();
    detail::MeshEntry e;
    e.n_cells = nC;
    check(mst_mesh_create(&d, &e.mesh));
    mst_params p = detail::default_params();
#if defined(ACCURACY)
    p.order = ACCURACY;
#endif
#if defined(RHOSOLVER)
    p.flux = std::is_same<RHOSOLVER, SolverAusm>::value ? MST_FLUX_AUSM : MST_FLUX_ROE;
#endif
    mst_status s = mst_ctx_create(e.mesh, &p, &e.ctx);
    if (s != MST_OK) {
      mst_mesh_destroy(e.mesh);
      check(s);
    }
    return e;
  }

  MshBlockT* mesh_;
  std::fstream* log_;
  AllDataT* data_;
  double dt_;
  detail::MeshEntry* entry_;
};

}  // namespace mstcfd

// With the reference's headers in scope (MshBlock, AllData and the VCTDIMU
// macro of include/CONST.h), GpuRhoSolver is the drop-in class.
#if defined(VCTDIMU)
typedef mstcfd::GpuRhoSolverT<MshBlock, AllData, VCTDIMU> GpuRhoSolver;
#endif
