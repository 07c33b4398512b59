/*
 * ORACLE — test infrastructure only.  C entry points over the reference's
 * own CIC header (lib/parops_fast.h of maurorigo/JERALD), compiled from the
 * reference's source where it lies by oracle/build.py into
 * oracle/_ref/libjldref.so, with oracle/ref_stub/mpi.h standing in for MPI
 * at world size one.  Tests use it to pin oracle/cic_oracle.c and to make
 * the hash fixtures of tests/golden/ref_hashes.json.  Nothing in the product
 * links or calls this file.
 *
 * Each entry point follows the reference's XLA custom-call wrapper for the
 * same op at world size one (lib/cpu.cc:54-136): the edges are [0, N) on
 * every axis, positions are in mesh units, float pairs with int32 mesh
 * sizes and double with int64 (lib/cpu.cc:276-285).  The readouts reach the
 * decomposition layout and exchanged positions the way the reference does:
 * a ppaint on the same positions stores them (lib/cpu.cc:76, 95), then
 * preadout / preadout3D reads them.
 */
#include <cstdint>
#include <vector>

#include "parops_fast.h"

using namespace parops_jax;

namespace {

template <typename T>
struct RefState {
  Layout layout;
  T* expos = nullptr;
  RefState() { initLayout(&layout, 1); }
};

template <typename T>
RefState<T>& state() {
  static RefState<T> s;
  return s;
}

template <typename T, typename intT>
void edges_of(const intT* nmesh, intT* ex, intT* ey, intT* ez) {
  ex[0] = 0; ex[1] = nmesh[0];
  ey[0] = 0; ey[1] = nmesh[1];
  ez[0] = 0; ez[1] = nmesh[2];
}

template <typename T, typename intT>
void paint(const T* pos_in, int64_t n, const T* mass_in, const intT* nmesh_in, T* out) {
  std::vector<T> pos(pos_in, pos_in + 3 * n), mass(mass_in, mass_in + n);
  intT nm[3] = {nmesh_in[0], nmesh_in[1], nmesh_in[2]};
  intT ex[2], ey[2], ez[2];
  edges_of<T, intT>(nm, ex, ey, ez);
  T* p = pos.data();
  T* m = mass.data();
  intT* nmp = nm;
  intT *exp_ = ex, *eyp = ey, *ezp = ez;
  bool use_layout = false;
  MPI_Comm comm = MPI_COMM_WORLD;
  RefState<T>& s = state<T>();
  ppaint<T, intT>(p, n, m, nmp, exp_, eyp, ezp, &out, &s.layout, &s.expos, use_layout, comm);
}

template <typename T, typename intT>
void readout(const T* pos, int64_t n, const T* field_in, const intT* nmesh_in, const T* box_in,
             int32_t vjpdim, T* out) {
  intT nm[3] = {nmesh_in[0], nmesh_in[1], nmesh_in[2]};
  int64_t cells = (int64_t)nm[0] * nm[1] * nm[2];
  std::vector<T> scratch(cells), ones(n, (T)1), field(field_in, field_in + cells);
  paint<T, intT>(pos, n, ones.data(), nm, scratch.data());
  T box[3] = {box_in[0], box_in[1], box_in[2]};
  intT ex[2], ey[2], ez[2];
  edges_of<T, intT>(nm, ex, ey, ez);
  T* f = field.data();
  T* b = box;
  intT* nmp = nm;
  intT *exp_ = ex, *eyp = ey, *ezp = ez;
  MPI_Comm comm = MPI_COMM_WORLD;
  RefState<T>& s = state<T>();
  preadout<T, intT>(s.layout, s.expos, n, f, nmp, b, exp_, eyp, ezp, &out, comm, vjpdim);
}

template <typename T, typename intT>
void paint3d(const T* pos_in, int64_t n, const T* mass_in, const intT* nmesh_in, T* out) {
  std::vector<T> pos(pos_in, pos_in + 3 * n), mass(mass_in, mass_in + 3 * n);
  intT nm[3] = {nmesh_in[0], nmesh_in[1], nmesh_in[2]};
  intT ex[2], ey[2], ez[2];
  edges_of<T, intT>(nm, ex, ey, ez);
  T* p = pos.data();
  T* m = mass.data();
  intT* nmp = nm;
  intT *exp_ = ex, *eyp = ey, *ezp = ez;
  MPI_Comm comm = MPI_COMM_WORLD;
  RefState<T>& s = state<T>();
  ppaint3D<T, intT>(p, n, m, nmp, exp_, eyp, ezp, &out, &s.layout, &s.expos, comm);
}

template <typename T, typename intT>
void readout3d(const T* pos, int64_t n, const T* field_in, const intT* nmesh_in, const T* box_in,
               bool vjp, T* out) {
  intT nm[3] = {nmesh_in[0], nmesh_in[1], nmesh_in[2]};
  int64_t cells = (int64_t)nm[0] * nm[1] * nm[2];
  int64_t fcells = vjp ? cells : 3 * cells;
  std::vector<T> scratch(cells), ones(n, (T)1), field(field_in, field_in + fcells);
  paint<T, intT>(pos, n, ones.data(), nm, scratch.data());
  T box[3] = {box_in[0], box_in[1], box_in[2]};
  intT ex[2], ey[2], ez[2];
  edges_of<T, intT>(nm, ex, ey, ez);
  T* f = field.data();
  T* b = box;
  intT* nmp = nm;
  intT *exp_ = ex, *eyp = ey, *ezp = ez;
  MPI_Comm comm = MPI_COMM_WORLD;
  RefState<T>& s = state<T>();
  preadout3D<T, intT>(s.layout, s.expos, n, f, nmp, b, exp_, eyp, ezp, &out, comm, vjp);
}

}  // namespace

extern "C" {

void jref_ppaint_f32(const float* pos, int64_t n, const float* mass, const int32_t* nmesh, float* out) {
  paint<float, int32_t>(pos, n, mass, nmesh, out);
}
void jref_ppaint_f64(const double* pos, int64_t n, const double* mass, const int64_t* nmesh, double* out) {
  paint<double, int64_t>(pos, n, mass, nmesh, out);
}
void jref_preadout_f32(const float* pos, int64_t n, const float* field, const int32_t* nmesh,
                       const float* box, int32_t vjpdim, float* out) {
  readout<float, int32_t>(pos, n, field, nmesh, box, vjpdim, out);
}
void jref_preadout_f64(const double* pos, int64_t n, const double* field, const int64_t* nmesh,
                       const double* box, int32_t vjpdim, double* out) {
  readout<double, int64_t>(pos, n, field, nmesh, box, vjpdim, out);
}
void jref_ppaint3d_f32(const float* pos, int64_t n, const float* mass3, const int32_t* nmesh, float* out) {
  paint3d<float, int32_t>(pos, n, mass3, nmesh, out);
}
void jref_ppaint3d_f64(const double* pos, int64_t n, const double* mass3, const int64_t* nmesh, double* out) {
  paint3d<double, int64_t>(pos, n, mass3, nmesh, out);
}
void jref_preadout3d_f32(const float* pos, int64_t n, const float* field, const int32_t* nmesh,
                         const float* box, int32_t vjp, float* out) {
  readout3d<float, int32_t>(pos, n, field, nmesh, box, vjp != 0, out);
}
void jref_preadout3d_f64(const double* pos, int64_t n, const double* field, const int64_t* nmesh,
                         const double* box, int32_t vjp, double* out) {
  readout3d<double, int64_t>(pos, n, field, nmesh, box, vjp != 0, out);
}

}  // extern "C"
