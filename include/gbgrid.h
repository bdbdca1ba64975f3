/* gbgrid.h -- Grid-shaped C++ adapter over the C ABI of gbdwf.h (header only).
 *
 * Code written against Grid's fermion-operator path compiles against these classes
 * unchanged for that path: grids from SpaceTimeGrid, LatticeFermion / LatticeGaugeField,
 * WilsonFermion / MobiusFermion (FermionOperator interface), MdagMLinearOperator,
 * SchurDiagMooeeOperator, ConjugateGradient, ConjugateGradientReliableUpdate,
 * ConjugateGradientMultiShift, SchurRedBlackDiagMooeeSolve, ZMobiusFermion, MADWF with the
 * Pauli-Villars solvers, plus norm2 / innerProduct / axpy / axpby / axpy_norm /
 * pickCheckerboard / setCheckerboard / precisionChange / InsertSlice / ExtractSlice.  Every call forwards to the C ABI;
 * the fields live in device memory.  Reference interfaces:
 *   Grid/qcd/action/fermion/FermionOperator.h:40-192, MobiusFermion.h:45-56,
 *   WilsonFermion.h:139-142, Grid/algorithms/LinearOperator.h:44-105,286-349,590-616,
 *   Grid/algorithms/iterative/ConjugateGradient.h:55-257, ConjugateGradientReliableUpdate.h,
 *   SchurRedBlack.h:373-436, Grid/qcd/utils/SpaceTimeGrid.cc:49-80.
 *
 * Differences from Grid, by design:
 *   - errors throw Grid::GridError carrying the C status (Grid asserts);
 *   - fields of one geometry (4D extents, Ls) are created through one hidden "context"
 *     operator of that geometry, so they work with every operator built on their grid;
 *     all adapter objects share one non-blocking stream, so their work is ordered;
 *   - random fields come from the library's seeded generators (Grid's RNG streams
 *     cannot be reproduced); gaussian() draws N(0,1) per real component;
 *   - single process, single GPU: no MPI decomposition (simd / mpi layouts are accepted
 *     and ignored).
 */
#ifndef GBGRID_H
#define GBGRID_H

#ifndef __cplusplus
#error "gbgrid.h is C++; C callers use gbdwf.h"
#endif

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "gbdwf.h"

namespace Grid {

typedef double RealD;
typedef float RealF;
typedef RealD Real;
typedef std::complex<double> ComplexD;
typedef ComplexD Complex;
typedef int32_t Integer;
typedef std::vector<int> Coordinate;

enum { Even = 0, Odd = 1 };
enum { DaggerNo = 0, DaggerYes = 1 };
static constexpr int Nd = 4, Nc = 3, Ns = 4;
struct Zero {};

class GridError : public std::runtime_error {
 public:
  int status;
  GridError(int st, const std::string& msg) : std::runtime_error(msg), status(st) {}
};

namespace gbdetail {
inline void check(int rc, const char* what) {
  if (rc != GB_OK) {
    const char* e = gb_last_error();
    throw GridError(rc, std::string(what) + ": " + (e && *e ? e : gb_status_string(rc)));
  }
}
// the stream shared by every operator and field of the adapter
inline void* stream() {
  static void* s = [] {
    void* p = nullptr;
    check(gb_stream_create(&p), "gb_stream_create");
    return p;
  }();
  return s;
}
// One operator per geometry creates the device fields of every grid with that geometry.
// It is never destroyed: grids, like Grid's, live until the process ends.
inline gb_op_t context(const Coordinate& d4, int Ls) {
  static std::mutex m;
  static auto* reg = new std::map<std::vector<int>, gb_op_t>();
  std::lock_guard<std::mutex> lk(m);
  std::vector<int> key(d4);
  key.push_back(Ls);
  auto it = reg->find(key);
  if (it != reg->end()) return it->second;
  gb_op_t op = nullptr;
  if (Ls == 1) check(gb_wilson_create(d4.data(), 0.0, nullptr, GB_F32, 1, stream(), 0, &op), "gb_wilson_create");
  else check(gb_mobius_create(d4.data(), Ls, 0.0, 1.0, 1.0, 0.0, nullptr, GB_F32, 1, stream(), 0, &op), "gb_mobius_create");
  (*reg)[key] = op;
  return op;
}
}  // namespace gbdetail

// ---- grids (Grid/cartesian/Cartesian_full.h, Cartesian_red_black.h) ------------------
class GridBase {
 public:
  Coordinate _fdimensions;  // full extents; a 5D grid lists s first, as Grid does
  Coordinate _gdimensions;  // checkerboarded grids halve x
  int _ndimension = 4;
  int _isCheckerBoarded = 0;
  int Ls = 1;               // 1 on 4D grids
  Coordinate dims4;         // the 4D extents
  virtual ~GridBase() {}
  int Nd() const { return _ndimension; }
  const Coordinate& FullDimensions() const { return _fdimensions; }
  const Coordinate& GlobalDimensions() const { return _gdimensions; }
  int64_t gSites() const {
    int64_t n = 1;
    for (int d : _gdimensions) n *= d;
    return n;
  }
  int64_t lSites() const { return gSites(); }
  gb_op_t context() const { return gbdetail::context(dims4, Ls); }

 protected:
  void init(const Coordinate& d4, int ls, int cb) {
    dims4 = d4;
    Ls = ls;
    _isCheckerBoarded = cb;
    _fdimensions.clear();
    if (ls > 1) _fdimensions.push_back(ls);
    for (int d : d4) _fdimensions.push_back(d);
    _ndimension = int(_fdimensions.size());
    _gdimensions = _fdimensions;
    if (cb) _gdimensions[ls > 1 ? 1 : 0] /= 2;
  }
};
class GridCartesian : public GridBase {
 public:
  explicit GridCartesian(const Coordinate& d4, int ls = 1) { init(d4, ls, 0); }
};
class GridRedBlackCartesian : public GridBase {
 public:
  explicit GridRedBlackCartesian(const GridBase* base) { init(base->dims4, base->Ls, 1); }
};

inline Coordinate GridDefaultSimd(int nd, int) { return Coordinate(nd, 1); }
inline Coordinate GridDefaultMpi() { return Coordinate(4, 1); }

// SpaceTimeGrid (Grid/qcd/utils/SpaceTimeGrid.cc:49-80); the caller owns the grids
namespace SpaceTimeGrid {
inline GridCartesian* makeFourDimGrid(const Coordinate& latt, const Coordinate& = Coordinate(),
                                      const Coordinate& = Coordinate()) {
  if (latt.size() != 4) throw GridError(GB_ERR_BAD_ARG, "makeFourDimGrid: 4 extents expected");
  return new GridCartesian(latt);
}
inline GridRedBlackCartesian* makeFourDimRedBlackGrid(const GridCartesian* g) { return new GridRedBlackCartesian(g); }
inline GridCartesian* makeFiveDimGrid(int Ls, const GridCartesian* g) { return new GridCartesian(g->dims4, Ls); }
inline GridRedBlackCartesian* makeFiveDimRedBlackGrid(int Ls, const GridCartesian* g) {
  GridCartesian full(g->dims4, Ls);
  return new GridRedBlackCartesian(&full);
}
}  // namespace SpaceTimeGrid

// ---- fields --------------------------------------------------------------------------
struct vSpinColourVectorD { static constexpr int precision = GB_F64; };
struct vSpinColourVectorF { static constexpr int precision = GB_F32; };
// FP16 storage with per-site FP32 norms (no Grid counterpart: Grid keeps half precision
// for halo messages only)
struct vSpinColourVectorH { static constexpr int precision = GB_F16; };
struct vLorentzColourMatrixD {};
struct vLorentzColourMatrixF {};

// Checkerboard() of a field: readable as an int and assignable, like Grid's int&
class CheckerboardRef {
  gb_field_t h_;

 public:
  explicit CheckerboardRef(gb_field_t h) : h_(h) {}
  operator int() const {
    int s = 0;
    gbdetail::check(gb_field_subset(h_, &s), "gb_field_subset");
    return s == GB_FULL ? Even : s;
  }
  CheckerboardRef& operator=(int cb) {
    int s = 0;
    gbdetail::check(gb_field_subset(h_, &s), "gb_field_subset");
    if (s != GB_FULL) gbdetail::check(gb_field_set_subset(h_, cb), "gb_field_set_subset");
    return *this;
  }
};

// A fermion field in device memory on a 4D or 5D, full or red-black grid.
template <class vobj> class Lattice {
  GridBase* grid_ = nullptr;
  gb_field_t h_ = nullptr;
  bool owned_ = true;
  Lattice(GridBase* grid, gb_field_t h, bool owned) : grid_(grid), h_(h), owned_(owned) {}

 public:
  typedef vobj vector_object;
  explicit Lattice(GridBase* grid) : grid_(grid) {
    gbdetail::check(gb_field_create(grid->context(), grid->_isCheckerBoarded ? GB_EVEN : GB_FULL, vobj::precision, &h_),
                    "gb_field_create");
  }
  // a Lattice over a field that the library owns (the work fields MADWF hands to the
  // solvers it calls back); it never destroys the field
  static Lattice View(GridBase* grid, gb_field_t h) { return Lattice(grid, h, false); }
  Lattice(const Lattice& o) : Lattice(o.grid_) { *this = o; }
  Lattice(Lattice&& o) noexcept : grid_(o.grid_), h_(o.h_), owned_(o.owned_) { o.h_ = nullptr; }
  ~Lattice() {
    if (h_ && owned_) gb_field_destroy(h_);
  }
  Lattice& operator=(const Lattice& o) {
    if (this != &o) gbdetail::check(gb_field_copy(h_, o.h_), "gb_field_copy");
    return *this;
  }
  Lattice& operator=(Lattice&& o) noexcept {
    std::swap(grid_, o.grid_);
    std::swap(h_, o.h_);
    std::swap(owned_, o.owned_);
    return *this;
  }
  Lattice& operator=(const Zero&) {
    gbdetail::check(gb_field_zero(h_), "gb_field_zero");
    return *this;
  }
  GridBase* Grid() const { return grid_; }
  CheckerboardRef Checkerboard() const { return CheckerboardRef(h_); }
  gb_field_t handle() const { return h_; }
  // canonical host form (complex per site, s, spin, colour; one checkerboard's sites in
  // lexicographic order for red-black fields) -- Grid's vectorizeFromLexOrdArray
  size_t HostSize() const {
    size_t n = 0;
    gbdetail::check(gb_field_host_len(h_, &n), "gb_field_host_len");
    return n / 2;
  }
  void ImportHost(const std::vector<ComplexD>& v) {
    if (v.size() != HostSize()) throw GridError(GB_ERR_BAD_ARG, "ImportHost: wrong size");
    gbdetail::check(gb_field_import(h_, reinterpret_cast<const double*>(v.data())), "gb_field_import");
  }
  std::vector<ComplexD> ExportHost() const {
    std::vector<ComplexD> v(HostSize());
    gbdetail::check(gb_field_export(h_, reinterpret_cast<double*>(v.data())), "gb_field_export");
    return v;
  }
};

typedef Lattice<vSpinColourVectorD> LatticeFermionD;
typedef Lattice<vSpinColourVectorF> LatticeFermionF;
typedef Lattice<vSpinColourVectorH> LatticeFermionH;
typedef LatticeFermionD LatticeFermion;

// The gauge field stays on the host in canonical form U[site][mu][3][3]; operators copy
// it to the device in ImportGauge.
template <class Tag> class GaugeLattice {
  GridBase* grid_;

 public:
  std::vector<ComplexD> data;
  explicit GaugeLattice(GridBase* grid) : grid_(grid), data(size_t(grid->gSites()) * Nd * Nc * Nc) {}
  GridBase* Grid() const { return grid_; }
  template <class T2> GaugeLattice& operator=(const GaugeLattice<T2>& o) {
    data = o.data;
    return *this;
  }
};
typedef GaugeLattice<vLorentzColourMatrixD> LatticeGaugeFieldD;
typedef GaugeLattice<vLorentzColourMatrixF> LatticeGaugeFieldF;
typedef LatticeGaugeFieldD LatticeGaugeField;

// ---- field linear algebra (Grid/lattice/Lattice_arith.h, Lattice_reduction.h) --------
template <class v> RealD norm2(const Lattice<v>& x) {
  double n = 0;
  gbdetail::check(gb_field_norm2(x.handle(), &n), "gb_field_norm2");
  return n;
}
template <class v> ComplexD innerProduct(const Lattice<v>& a, const Lattice<v>& b) {
  double r[2] = {0, 0};
  gbdetail::check(gb_field_inner(a.handle(), b.handle(), r), "gb_field_inner");
  return ComplexD(r[0], r[1]);
}
inline double real_coeff(ComplexD a) {
  if (a.imag() != 0) throw GridError(GB_ERR_UNSUPPORTED, "complex field coefficients are not supported");
  return a.real();
}
template <class v> void axpy(Lattice<v>& ret, ComplexD a, const Lattice<v>& x, const Lattice<v>& y) {
  gbdetail::check(gb_field_axpy(ret.handle(), real_coeff(a), x.handle(), y.handle()), "gb_field_axpy");
}
template <class v> void axpby(Lattice<v>& ret, ComplexD a, ComplexD b, const Lattice<v>& x, const Lattice<v>& y) {
  gbdetail::check(gb_field_axpby(ret.handle(), real_coeff(a), real_coeff(b), x.handle(), y.handle()), "gb_field_axpby");
}
template <class v> RealD axpy_norm(Lattice<v>& ret, ComplexD a, const Lattice<v>& x, const Lattice<v>& y) {
  double n = 0;
  gbdetail::check(gb_field_axpy_norm(ret.handle(), real_coeff(a), x.handle(), y.handle(), &n), "gb_field_axpy_norm");
  return n;
}
template <class v> RealD axpby_norm(Lattice<v>& ret, ComplexD a, ComplexD b, const Lattice<v>& x, const Lattice<v>& y) {
  double n = 0;
  gbdetail::check(gb_field_axpby_norm(ret.handle(), real_coeff(a), real_coeff(b), x.handle(), y.handle(), &n),
                  "gb_field_axpby_norm");
  return n;
}
template <class v> void innerProductNorm(ComplexD& ip, RealD& nrm, const Lattice<v>& left, const Lattice<v>& right) {
  double r[2] = {0, 0}, n = 0;
  gbdetail::check(gb_field_inner_norm(left.handle(), right.handle(), r, &n), "gb_field_inner_norm");
  ip = ComplexD(r[0], r[1]);
  nrm = n;
}
// one process, one GPU: the rank-local inner product is the global one
template <class v> ComplexD rankInnerProduct(const Lattice<v>& a, const Lattice<v>& b) { return innerProduct(a, b); }
template <class v> void pickCheckerboard(int cb, Lattice<v>& half, const Lattice<v>& full) {
  half.Checkerboard() = cb;
  gbdetail::check(gb_field_pick_checkerboard(half.handle(), full.handle()), "gb_field_pick_checkerboard");
}
template <class v> void setCheckerboard(Lattice<v>& full, const Lattice<v>& half) {
  gbdetail::check(gb_field_set_checkerboard(full.handle(), half.handle()), "gb_field_set_checkerboard");
}
template <class vo, class vi> void precisionChange(Lattice<vo>& out, const Lattice<vi>& in) {
  gbdetail::check(gb_field_copy(out.handle(), in.handle()), "gb_field_copy");
}
template <class T1, class T2> void precisionChange(GaugeLattice<T1>& out, const GaugeLattice<T2>& in) {
  out.data = in.data;
}
// a - b, a + b and scalar * a as new fields (Grid's expression templates, evaluated eagerly)
template <class v> Lattice<v> operator-(const Lattice<v>& a, const Lattice<v>& b) {
  Lattice<v> r(a.Grid());
  axpby(r, 1.0, -1.0, a, b);
  return r;
}
template <class v> Lattice<v> operator+(const Lattice<v>& a, const Lattice<v>& b) {
  Lattice<v> r(a.Grid());
  axpby(r, 1.0, 1.0, a, b);
  return r;
}
template <class v> Lattice<v> operator*(RealD s, const Lattice<v>& a) {
  Lattice<v> r(a.Grid());
  axpby(r, s, 0.0, a, a);
  return r;
}
template <class v> Lattice<v> operator-(const Lattice<v>& a) { return -1.0 * a; }

// InsertSlice / ExtractSlice along the fifth dimension (Grid/lattice/Lattice_transfer.h:
// 999-1070; orthog = 0 is s on Grid's 5D grids): lowDim on a full 4D grid, higherDim on a
// full 5D grid with the same 4D extents
namespace gbdetail {
inline void check_slice_grids(const GridBase* low, const GridBase* high, int orthog, const char* what) {
  if (orthog != 0) throw GridError(GB_ERR_UNSUPPORTED, std::string(what) + ": only orthog = 0 (the fifth dimension)");
  if (low->Ls != 1 || low->_isCheckerBoarded || high->Ls < 2 || high->_isCheckerBoarded || low->dims4 != high->dims4)
    throw GridError(GB_ERR_BAD_ARG, std::string(what) + ": a full 4D and a full 5D field of the same extents expected");
}
}  // namespace gbdetail
template <class v> void InsertSlice(const Lattice<v>& lowDim, Lattice<v>& higherDim, int slice, int orthog) {
  gbdetail::check_slice_grids(lowDim.Grid(), higherDim.Grid(), orthog, "InsertSlice");
  const std::vector<ComplexD> h = lowDim.ExportHost();
  gbdetail::check(gb_insert_slice(higherDim.Grid()->context(), reinterpret_cast<const double*>(h.data()), 0,
                                  higherDim.handle(), slice),
                  "InsertSlice");
}
template <class v> void ExtractSlice(Lattice<v>& lowDim, const Lattice<v>& higherDim, int slice, int orthog) {
  gbdetail::check_slice_grids(lowDim.Grid(), higherDim.Grid(), orthog, "ExtractSlice");
  std::vector<ComplexD> h(lowDim.HostSize());
  gbdetail::check(gb_extract_slice(higherDim.Grid()->context(), higherDim.handle(), slice,
                                   reinterpret_cast<double*>(h.data()), 0),
                  "ExtractSlice");
  lowDim.ImportHost(h);
}
// MADWF.h:33-42: a copy that changes precision when the field types differ
template <class vi, class vo> void convert(const Lattice<vi>& from, Lattice<vo>& to) { precisionChange(to, from); }

// ---- seeded synthetic inputs (GridParallelRNG + gaussian + SU3 configurations) --------
class GridParallelRNG {
  uint64_t seed_ = 0x9E3779B97F4A7C15ull, draws_ = 0;

 public:
  explicit GridParallelRNG(GridBase*) {}
  void SeedFixedIntegers(const std::vector<int>& seeds) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the seed integers
    for (int s : seeds) {
      for (int k = 0; k < 4; k++) {
        h ^= uint64_t((uint32_t(s) >> (8 * k)) & 0xff);
        h *= 1099511628211ull;
      }
    }
    seed_ = h;
    draws_ = 0;
  }
  uint64_t next() { return seed_ + 0x632BE59BD9B4E019ull * ++draws_; }
};
template <class v> void gaussian(GridParallelRNG& rng, Lattice<v>& f) {
  std::vector<ComplexD> buf(f.HostSize());
  gbdetail::check(gb_random_gaussian(buf.size(), rng.next(), reinterpret_cast<double*>(buf.data())), "gb_random_gaussian");
  f.ImportHost(buf);
}
template <class v> void random(GridParallelRNG& rng, Lattice<v>& f) { gaussian(rng, f); }

template <int N> struct SU {
  static_assert(N == 3, "SU(3) only");
  // U = exp(i eps H), H traceless Hermitian with N(0,1) entries, reunitarised
  template <class T> static void ExpiHConfiguration(GridParallelRNG& rng, GaugeLattice<T>& U, RealD eps) {
    gbdetail::check(gb_random_gauge(U.Grid()->dims4.data(), eps, rng.next(), reinterpret_cast<double*>(U.data.data())),
                    "gb_random_gauge");
  }
  template <class T> static void HotConfiguration(GridParallelRNG& rng, GaugeLattice<T>& U) {
    ExpiHConfiguration(rng, U, 1.0);
  }
  template <class T> static void TepidConfiguration(GridParallelRNG& rng, GaugeLattice<T>& U) {
    ExpiHConfiguration(rng, U, 0.01);
  }
  template <class T> static void ColdConfiguration(GaugeLattice<T>& U) {
    gbdetail::check(gb_unit_gauge(U.Grid()->dims4.data(), reinterpret_cast<double*>(U.data.data())), "gb_unit_gauge");
  }
  template <class T> static void ColdConfiguration(GridParallelRNG&, GaugeLattice<T>& U) { ColdConfiguration(U); }
};
typedef SU<3> SU3;

// ---- fermion operators (FermionOperator.h:40-192) ------------------------------------
struct WilsonImplParams {
  std::vector<ComplexD> boundary_phases = std::vector<ComplexD>(Nd, ComplexD(1, 0));
  // this library's operator options (not in Grid): GB_FLAG_RECON12 (12-real links),
  // GB_FLAG_DF64 (FP64 operators: the hopping term in double-float arithmetic)
  unsigned flags = 0;
  WilsonImplParams() {}
  explicit WilsonImplParams(const std::vector<ComplexD>& phi) : boundary_phases(phi) {}
};
template <class vobj, class GaugeTag> struct WilsonImplT {
  typedef Lattice<vobj> FermionField;
  typedef GaugeLattice<GaugeTag> GaugeField;
  typedef WilsonImplParams ImplParams;
  static constexpr int precision = vobj::precision;
};
typedef WilsonImplT<vSpinColourVectorD, vLorentzColourMatrixD> WilsonImplD;
typedef WilsonImplT<vSpinColourVectorF, vLorentzColourMatrixF> WilsonImplF;
typedef WilsonImplT<vSpinColourVectorH, vLorentzColourMatrixF> WilsonImplH;
typedef WilsonImplD WilsonImplR;

// CheckerBoardedSparseMatrixBase / FermionOperator<Impl>
template <class Impl> class FermionOperator {
 public:
  typedef typename Impl::FermionField FermionField;
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;

  FermionOperator(const FermionOperator&) = delete;
  FermionOperator& operator=(const FermionOperator&) = delete;
  virtual ~FermionOperator() {
    if (op_) gb_op_destroy(op_);
  }
  gb_op_t handle() const { return op_; }
  GridBase* FermionGrid() const { return fgrid_; }
  GridBase* FermionRedBlackGrid() const { return frbgrid_; }
  GridBase* GaugeGrid() const { return ugrid_; }
  GridBase* GaugeRedBlackGrid() const { return urbgrid_; }
  RealD Mass() const { return mass_; }

  void ImportGauge(const GaugeField& U) {
    gbdetail::check(gb_op_import_gauge(op_, reinterpret_cast<const double*>(U.data.data())), "ImportGauge");
  }
  void M(const FermionField& in, FermionField& out) { run(gb_M(op_, in.handle(), out.handle()), "M"); }
  void Mdag(const FermionField& in, FermionField& out) { run(gb_Mdag(op_, in.handle(), out.handle()), "Mdag"); }
  void MdagM(const FermionField& in, FermionField& out) { run(gb_MdagM(op_, in.handle(), out.handle()), "MdagM"); }
  void Dhop(const FermionField& in, FermionField& out, int dag) {
    run(gb_Dhop(op_, in.handle(), out.handle(), dag), "Dhop");
  }
  void DhopEO(const FermionField& in, FermionField& out, int dag) {
    run(gb_DhopEO(op_, in.handle(), out.handle(), dag), "DhopEO");
  }
  void DhopOE(const FermionField& in, FermionField& out, int dag) {
    run(gb_DhopOE(op_, in.handle(), out.handle(), dag), "DhopOE");
  }
  void Meooe(const FermionField& in, FermionField& out) { run(gb_Meooe(op_, in.handle(), out.handle()), "Meooe"); }
  void MeooeDag(const FermionField& in, FermionField& out) {
    run(gb_MeooeDag(op_, in.handle(), out.handle()), "MeooeDag");
  }
  void Mooee(const FermionField& in, FermionField& out) { run(gb_Mooee(op_, in.handle(), out.handle()), "Mooee"); }
  void MooeeDag(const FermionField& in, FermionField& out) {
    run(gb_MooeeDag(op_, in.handle(), out.handle()), "MooeeDag");
  }
  void MooeeInv(const FermionField& in, FermionField& out) {
    run(gb_MooeeInv(op_, in.handle(), out.handle()), "MooeeInv");
  }
  void MooeeInvDag(const FermionField& in, FermionField& out) {
    run(gb_MooeeInvDag(op_, in.handle(), out.handle()), "MooeeInvDag");
  }
  // SchurDiagMooeeOperator's pieces (LinearOperator.h:325-349)
  void Mpc(const FermionField& in, FermionField& out) { run(gb_Mpc(op_, in.handle(), out.handle()), "Mpc"); }
  void MpcDag(const FermionField& in, FermionField& out) { run(gb_MpcDag(op_, in.handle(), out.handle()), "MpcDag"); }
  void MpcDagMpc(const FermionField& in, FermionField& out) {
    run(gb_MpcDagMpc(op_, in.handle(), out.handle()), "MpcDagMpc");
  }

 protected:
  gb_op_t op_ = nullptr;
  GridBase *fgrid_, *frbgrid_, *ugrid_, *urbgrid_;
  RealD mass_;
  FermionOperator(GridBase* f, GridBase* frb, GridBase* u, GridBase* urb, RealD mass)
      : fgrid_(f), frbgrid_(frb), ugrid_(u), urbgrid_(urb), mass_(mass) {}
  static std::vector<double> phases(const ImplParams& p) {
    std::vector<double> ph(2 * Nd);
    for (int k = 0; k < Nd; k++) {
      ph[2 * k] = p.boundary_phases[k].real();
      ph[2 * k + 1] = p.boundary_phases[k].imag();
    }
    return ph;
  }
  static void run(int rc, const char* what) { gbdetail::check(rc, what); }
};

// WilsonFermion(U, Fgrid, Hgrid, mass, ImplParams) (WilsonFermion.h:139-142)
template <class Impl> class WilsonFermion : public FermionOperator<Impl> {
  typedef FermionOperator<Impl> Base;

 public:
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;
  WilsonFermion(const GaugeField& U, GridCartesian& Fgrid, GridRedBlackCartesian& Hgrid, RealD mass,
                const ImplParams& p = ImplParams())
      : Base(&Fgrid, &Hgrid, &Fgrid, &Hgrid, mass) {
    const std::vector<double> ph = Base::phases(p);
    gbdetail::check(gb_wilson_create(Fgrid.dims4.data(), mass, ph.data(), Impl::precision, 1, gbdetail::stream(),
                                     p.flags, &this->op_),
                    "WilsonFermion");
    this->ImportGauge(U);
  }
};

// MobiusFermion(U, FGrid, FrbGrid, UGrid, UrbGrid, mf, M5, b, c, ImplParams)
// (MobiusFermion.h:45-56) with the CayleyFermion5D extras
template <class Impl> class MobiusFermion : public FermionOperator<Impl> {
  typedef FermionOperator<Impl> Base;

 public:
  typedef typename Impl::FermionField FermionField;
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;
  int Ls;
  RealD M5, b, c;
  ImplParams params;
  MobiusFermion(const GaugeField& U, GridCartesian& FiveDimGrid, GridRedBlackCartesian& FiveDimRedBlackGrid,
                GridCartesian& FourDimGrid, GridRedBlackCartesian& FourDimRedBlackGrid, RealD mass, RealD M5_,
                RealD b_, RealD c_, const ImplParams& p = ImplParams())
      : Base(&FiveDimGrid, &FiveDimRedBlackGrid, &FourDimGrid, &FourDimRedBlackGrid, mass),
        Ls(FiveDimGrid.Ls), M5(M5_), b(b_), c(c_), params(p) {
    const std::vector<double> ph = Base::phases(p);
    gbdetail::check(gb_mobius_create(FourDimGrid.dims4.data(), Ls, mass, M5_, b_, c_, ph.data(), Impl::precision, 1,
                                     gbdetail::stream(), p.flags, &this->op_),
                    "MobiusFermion");
    this->ImportGauge(U);
  }
  void Dminus(const FermionField& in, FermionField& out) {
    Base::run(gb_Dminus(this->op_, in.handle(), out.handle(), 0), "Dminus");
  }
  // MADWF support (CayleyFermion5D.h:71-85, CayleyFermion5DImplementation.h:70-88)
  void SetMass(RealD mass) {
    Base::run(gb_op_set_mass(this->op_, mass), "SetMass");
    this->mass_ = mass;
  }
  void P(const FermionField& psi, FermionField& chi) { Base::run(gb_P(this->op_, psi.handle(), chi.handle(), 0), "P"); }
  void Pdag(const FermionField& psi, FermionField& chi) {
    Base::run(gb_P(this->op_, psi.handle(), chi.handle(), 1), "Pdag");
  }
  void DminusDag(const FermionField& in, FermionField& out) {
    Base::run(gb_Dminus(this->op_, in.handle(), out.handle(), 1), "DminusDag");
  }
  // 4D <-> 5D surface fields (CayleyFermion5DImplementation.h:57-129); the 4D field is
  // any fermion field on the gauge grid
  template <class F4> void ImportPhysicalFermionSource(const F4& input4d, FermionField& imported5d) {
    const std::vector<ComplexD> v = input4d.ExportHost();
    Base::run(gb_import_physical_source(this->op_, reinterpret_cast<const double*>(v.data()), 0, imported5d.handle()),
              "ImportPhysicalFermionSource");
  }
  template <class F4> void ImportUnphysicalFermion(const F4& input4d, FermionField& imported5d) {
    const std::vector<ComplexD> v = input4d.ExportHost();
    Base::run(gb_import_unphysical_fermion(this->op_, reinterpret_cast<const double*>(v.data()), 0,
                                           imported5d.handle()),
              "ImportUnphysicalFermion");
  }
  template <class F4> void ExportPhysicalFermionSolution(const FermionField& solution5d, F4& exported4d) {
    std::vector<ComplexD> v(exported4d.HostSize());
    Base::run(gb_export_physical_solution(this->op_, solution5d.handle(), reinterpret_cast<double*>(v.data()), 0),
              "ExportPhysicalFermionSolution");
    exported4d.ImportHost(v);
  }
  template <class F4> void ExportPhysicalFermionSource(const FermionField& solution5d, F4& exported4d) {
    std::vector<ComplexD> v(exported4d.HostSize());
    Base::run(gb_export_physical_source(this->op_, solution5d.handle(), reinterpret_cast<double*>(v.data()), 0),
              "ExportPhysicalFermionSource");
    exported4d.ImportHost(v);
  }

 protected:
  // for derived operators that create the library operator themselves
  struct Deferred {};
  MobiusFermion(Deferred, GridCartesian& FiveDimGrid, GridRedBlackCartesian& FiveDimRedBlackGrid,
                GridCartesian& FourDimGrid, GridRedBlackCartesian& FourDimRedBlackGrid, RealD mass, RealD M5_,
                RealD b_, RealD c_)
      : Base(&FiveDimGrid, &FiveDimRedBlackGrid, &FourDimGrid, &FourDimRedBlackGrid, mass),
        Ls(FiveDimGrid.Ls), M5(M5_), b(b_), c(c_) {}
};

// ZMobiusFermion<Impl> (Grid/qcd/action/fermion/ZMobiusFermion.h:44-90): complex omega_s =
// gamma[s], bs = (b + c) omega_s / 2 + (b - c) / 2, cs = (b + c) omega_s / 2 - (b - c) / 2
// (FP64 and FP32 storage)
template <class Impl> class ZMobiusFermion : public MobiusFermion<Impl> {
  typedef MobiusFermion<Impl> Base;

 public:
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;
  std::vector<ComplexD> omega;
  ZMobiusFermion(const GaugeField& U, GridCartesian& FiveDimGrid, GridRedBlackCartesian& FiveDimRedBlackGrid,
                 GridCartesian& FourDimGrid, GridRedBlackCartesian& FourDimRedBlackGrid, RealD mass, RealD M5_,
                 const std::vector<ComplexD>& gamma, RealD b_, RealD c_, const ImplParams& p = ImplParams())
      : Base(typename Base::Deferred(), FiveDimGrid, FiveDimRedBlackGrid, FourDimGrid, FourDimRedBlackGrid, mass,
             M5_, b_, c_),
        omega(gamma) {
    if (int(gamma.size()) != this->Ls) throw GridError(GB_ERR_BAD_ARG, "ZMobiusFermion: gamma.size() != Ls");
    this->params = p;
    const std::vector<double> ph = FermionOperator<Impl>::phases(p);
    gbdetail::check(gb_zmobius_create(FourDimGrid.dims4.data(), this->Ls, mass, M5_,
                                      reinterpret_cast<const double*>(gamma.data()), b_, c_, ph.data(),
                                      Impl::precision, 1, gbdetail::stream(), p.flags, &this->op_),
                    "ZMobiusFermion");
    this->ImportGauge(U);
  }
};

typedef WilsonFermion<WilsonImplD> WilsonFermionD;
typedef WilsonFermion<WilsonImplF> WilsonFermionF;
typedef WilsonFermionD WilsonFermionR;
typedef MobiusFermion<WilsonImplD> MobiusFermionD;
typedef MobiusFermion<WilsonImplF> MobiusFermionF;
typedef MobiusFermion<WilsonImplH> MobiusFermionH;
typedef MobiusFermionD MobiusFermionR;

// ---- Approx::zolotarev / higham (Grid/algorithms/approx/Zolotarev.h): the fields the
// Cayley operators use (gamma, n, Delta, epsilon, type) ----------------------------------
namespace Approx {
struct zolotarev_data {
  double* gamma = nullptr;
  double Delta = 0, epsilon = 0;
  int n = 0, type = 0;
};
inline zolotarev_data* zolotarev(double epsilon, int n, int type) {
  zolotarev_data* z = new zolotarev_data;
  z->gamma = new double[n];
  z->n = n;
  z->type = type;
  z->epsilon = epsilon;
  const int rc = gb_zolotarev(epsilon, n, type, z->gamma, &z->Delta);
  if (rc != GB_OK) {
    delete[] z->gamma;
    delete z;
    gbdetail::check(rc, "Approx::zolotarev");
  }
  return z;
}
// the tanh approximation: every Cayley zero is 1 (Zolotarev.cc:429-531)
inline zolotarev_data* higham(double epsilon, int n) {
  zolotarev_data* z = new zolotarev_data;
  z->gamma = new double[n];
  for (int i = 0; i < n; i++) z->gamma[i] = 1.0;
  z->n = n;
  z->epsilon = epsilon;
  return z;
}
// Approx::computeZmobiusGamma (Grid/algorithms/approx/ZMobius.cc:149-175)
inline void computeZmobiusGamma(std::vector<ComplexD>& gamma_out, RealD mobius_param_out, int Ls_out,
                                RealD mobius_param_in, int Ls_in, RealD lambda_bound) {
  std::vector<double> g(2 * size_t(Ls_out));
  gbdetail::check(gb_zmobius_gamma(Ls_out, mobius_param_out, Ls_in, mobius_param_in, lambda_bound, g.data(), nullptr),
                  "Approx::computeZmobiusGamma");
  gamma_out.resize(Ls_out);
  for (int s = 0; s < Ls_out; s++) gamma_out[s] = ComplexD(g[2 * s], g[2 * s + 1]);
}
inline void computeZmobiusGamma(std::vector<ComplexD>& gamma_out, int Ls_out, RealD mobius_param, int Ls_in,
                                RealD lambda_bound) {
  computeZmobiusGamma(gamma_out, mobius_param, Ls_out, mobius_param, Ls_in, lambda_bound);
}
inline void zolotarev_free(zolotarev_data* z) {
  if (z) {
    delete[] z->gamma;
    delete z;
  }
}
}  // namespace Approx
// MobiusZolotarevFermion / ShamirZolotarevFermion (MobiusZolotarevFermion.h:45-70,
// ShamirZolotarevFermion.h): omega_s = hi * gamma_s of Approx::zolotarev(lo / hi, Ls, 0)
// (CayleyFermion5DImplementation.h:445-447), through the complex-coefficient operator
namespace gbdetail {
inline std::vector<ComplexD> zolotarev_omega(int Ls, RealD lo, RealD hi) {
  Approx::zolotarev_data* z = Approx::zolotarev(lo / hi, Ls, 0);
  std::vector<ComplexD> w(Ls);
  for (int s = 0; s < Ls; s++) w[s] = ComplexD(hi * z->gamma[s], 0.0);
  Approx::zolotarev_free(z);
  return w;
}
}  // namespace gbdetail
template <class Impl> class MobiusZolotarevFermion : public ZMobiusFermion<Impl> {
 public:
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;
  MobiusZolotarevFermion(const GaugeField& U, GridCartesian& FiveDimGrid, GridRedBlackCartesian& FiveDimRedBlackGrid,
                         GridCartesian& FourDimGrid, GridRedBlackCartesian& FourDimRedBlackGrid, RealD mass, RealD M5_,
                         RealD b_, RealD c_, RealD lo, RealD hi, const ImplParams& p = ImplParams())
      : ZMobiusFermion<Impl>(U, FiveDimGrid, FiveDimRedBlackGrid, FourDimGrid, FourDimRedBlackGrid, mass, M5_,
                             gbdetail::zolotarev_omega(FiveDimGrid.Ls, lo, hi), b_, c_, p) {}
};
template <class Impl> class ShamirZolotarevFermion : public MobiusZolotarevFermion<Impl> {
 public:
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;
  ShamirZolotarevFermion(const GaugeField& U, GridCartesian& FiveDimGrid, GridRedBlackCartesian& FiveDimRedBlackGrid,
                         GridCartesian& FourDimGrid, GridRedBlackCartesian& FourDimRedBlackGrid, RealD mass, RealD M5_,
                         RealD lo, RealD hi, const ImplParams& p = ImplParams())
      : MobiusZolotarevFermion<Impl>(U, FiveDimGrid, FiveDimRedBlackGrid, FourDimGrid, FourDimRedBlackGrid, mass, M5_,
                                     1.0, 0.0, lo, hi, p) {}
};
// ScaledShamirFermion (ScaledShamirFermion.h): Moebius with b + c = scale, b - c = 1
template <class Impl> class ScaledShamirFermion : public MobiusFermion<Impl> {
 public:
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;
  ScaledShamirFermion(const GaugeField& U, GridCartesian& FiveDimGrid, GridRedBlackCartesian& FiveDimRedBlackGrid,
                      GridCartesian& FourDimGrid, GridRedBlackCartesian& FourDimRedBlackGrid, RealD mass, RealD M5_,
                      RealD scale, const ImplParams& p = ImplParams())
      : MobiusFermion<Impl>(U, FiveDimGrid, FiveDimRedBlackGrid, FourDimGrid, FourDimRedBlackGrid, mass, M5_,
                            0.5 * (scale + 1.0), 0.5 * (scale - 1.0), p) {}
};

// WilsonTMFermion5D<Impl> (WilsonTMFermion5D.h:40-145): FiveDimGrid.Ls slices of the 4D
// Wilson hop with Mooee = (4 + mass[s]) + i mu[s] gamma5
template <class Impl> class WilsonTMFermion5D : public FermionOperator<Impl> {
  typedef FermionOperator<Impl> Base;

 public:
  typedef typename Impl::GaugeField GaugeField;
  typedef typename Impl::ImplParams ImplParams;
  WilsonTMFermion5D(const GaugeField& U, GridCartesian& FiveDimGrid, GridRedBlackCartesian& FiveDimRedBlackGrid,
                    GridCartesian& FourDimGrid, GridRedBlackCartesian& FourDimRedBlackGrid,
                    const std::vector<RealD>& mass, const std::vector<RealD>& mu, const ImplParams& p = ImplParams())
      : Base(&FiveDimGrid, &FiveDimRedBlackGrid, &FourDimGrid, &FourDimRedBlackGrid, 0.0) {
    if (int(mass.size()) != FiveDimGrid.Ls || mu.size() != mass.size())
      throw GridError(GB_ERR_BAD_ARG, "WilsonTMFermion5D: one mass and one mu per slice");
    const std::vector<double> ph = Base::phases(p);
    gbdetail::check(gb_wilson_tm5d_create(FourDimGrid.dims4.data(), FiveDimGrid.Ls, mass.data(), mu.data(), ph.data(),
                                          Impl::precision, gbdetail::stream(), 0, &this->op_),
                    "WilsonTMFermion5D");
    this->ImportGauge(U);
  }
  void update(const std::vector<RealD>& mass, const std::vector<RealD>& mu) {
    Base::run(gb_op_tm_update(this->op_, mass.data(), mu.data()), "WilsonTMFermion5D::update");
  }
};

// Grid's ZWilsonImpl carries the complex Cayley coefficients in the action; here the
// operator does, so the implementation tags are the Wilson ones
typedef WilsonImplD ZWilsonImplD;
typedef WilsonImplF ZWilsonImplF;
typedef ZMobiusFermion<ZWilsonImplD> ZMobiusFermionD;
typedef ZMobiusFermion<ZWilsonImplF> ZMobiusFermionF;
typedef ZMobiusFermionD ZMobiusFermionR;
typedef MobiusZolotarevFermion<WilsonImplD> MobiusZolotarevFermionD;
typedef MobiusZolotarevFermion<WilsonImplF> MobiusZolotarevFermionF;
typedef ShamirZolotarevFermion<WilsonImplD> ShamirZolotarevFermionD;
typedef ShamirZolotarevFermion<WilsonImplF> ShamirZolotarevFermionF;
typedef ScaledShamirFermion<WilsonImplD> ScaledShamirFermionD;
typedef ScaledShamirFermion<WilsonImplF> ScaledShamirFermionF;

// ---- linear operators (Grid/algorithms/LinearOperator.h:44-105,286-349) --------------
template <class Field> class LinearOperatorBase {
 public:
  virtual ~LinearOperatorBase() {}
  virtual void Op(const Field& in, Field& out) = 0;
  virtual void AdjOp(const Field& in, Field& out) = 0;
  virtual void HermOp(const Field& in, Field& out) = 0;
  virtual void HermOpAndNorm(const Field& in, Field& out, RealD& n1, RealD& n2) {
    HermOp(in, out);
    const ComplexD dot = innerProduct(in, out);
    n1 = dot.real();
    n2 = norm2(out);
  }
  virtual void OpDiag(const Field&, Field&) { throw GridError(GB_ERR_UNSUPPORTED, "OpDiag"); }
  virtual void OpDir(const Field&, Field&, int, int) { throw GridError(GB_ERR_UNSUPPORTED, "OpDir"); }
  virtual void OpDirAll(const Field&, std::vector<Field>&) { throw GridError(GB_ERR_UNSUPPORTED, "OpDirAll"); }
  // the library operator behind this linear operator and its kind (0 MdagM, 1 Schur), or
  // null for a user-defined operator (solved by the host-driven CG below)
  virtual gb_op_t library_op() const { return nullptr; }
  virtual int library_kind() const { return -1; }
};

template <class Matrix, class Field> class MdagMLinearOperator : public LinearOperatorBase<Field> {
  Matrix& _Mat;

 public:
  explicit MdagMLinearOperator(Matrix& Mat) : _Mat(Mat) {}
  void Op(const Field& in, Field& out) override { _Mat.M(in, out); }
  void AdjOp(const Field& in, Field& out) override { _Mat.Mdag(in, out); }
  void HermOp(const Field& in, Field& out) override { _Mat.MdagM(in, out); }
  gb_op_t library_op() const override { return _Mat.handle(); }
  int library_kind() const override { return 0; }
};

template <class Matrix, class Field> class SchurDiagMooeeOperator : public LinearOperatorBase<Field> {
  Matrix& _Mat;

 public:
  explicit SchurDiagMooeeOperator(Matrix& Mat) : _Mat(Mat) {}
  void Mpc(const Field& in, Field& out) { _Mat.Mpc(in, out); }
  void MpcDag(const Field& in, Field& out) { _Mat.MpcDag(in, out); }
  void MpcDagMpc(const Field& in, Field& out) { _Mat.MpcDagMpc(in, out); }
  void Op(const Field& in, Field& out) override { Mpc(in, out); }
  void AdjOp(const Field& in, Field& out) override { MpcDag(in, out); }
  void HermOp(const Field& in, Field& out) override { MpcDagMpc(in, out); }
  gb_op_t library_op() const override { return _Mat.handle(); }
  int library_kind() const override { return 1; }
};

// ---- solvers ---------------------------------------------------------------------------
template <class Field> class OperatorFunction {
 public:
  virtual ~OperatorFunction() {}
  virtual void operator()(LinearOperatorBase<Field>& Linop, const Field& in, Field& out) = 0;
};
template <class Field> class LinearFunction {
 public:
  virtual ~LinearFunction() {}
  virtual void operator()(const Field& in, Field& out) = 0;
};

// ConjugateGradient<Field>(tol, maxit, err_on_no_conv) (ConjugateGradient.h:55-257).  A
// library operator runs the device-resident CG of the C ABI; any other linear operator
// runs Grid's iteration driven from the host over the device field algebra.
template <class Field> class ConjugateGradient : public OperatorFunction<Field> {
 public:
  RealD Tolerance;
  Integer MaxIterations;
  bool ErrorOnNoConverge;
  Integer IterationsToComplete = 0;
  RealD TrueResidual = 0;
  bool UseGraphs = false;  // capture iteration chunks as CUDA graphs
  ConjugateGradient(RealD tol, Integer maxit, bool err_on_no_conv = true)
      : Tolerance(tol), MaxIterations(maxit), ErrorOnNoConverge(err_on_no_conv) {}

  gb_cg_params params() const {
    gb_cg_params p;
    gb_cg_params_default(&p);
    p.tolerance = Tolerance;
    p.max_iterations = MaxIterations;
    p.err_on_no_conv = ErrorOnNoConverge ? 1 : 0;
    p.use_graphs = UseGraphs ? 1 : 0;
    return p;
  }
  void operator()(LinearOperatorBase<Field>& Linop, const Field& src, Field& psi) override {
    if (gb_op_t op = Linop.library_op()) {
      const gb_cg_params p = params();
      gb_cg_result r;
      const int rc = Linop.library_kind() == 1 ? gb_cg_schur(op, src.handle(), psi.handle(), &p, &r)
                                               : gb_cg_mdagm(op, src.handle(), psi.handle(), &p, &r);
      IterationsToComplete = r.iterations;
      TrueResidual = r.true_residual;
      gbdetail::check(rc, "ConjugateGradient");
      return;
    }
    generic(Linop, src, psi);
  }

 private:
  // ConjugateGradient.h:68-257, with every vector operation on the device
  void generic(LinearOperatorBase<Field>& Linop, const Field& src, Field& psi) {
    Field p(src.Grid()), mmp(src.Grid()), r(src.Grid());
    p.Checkerboard() = int(src.Checkerboard());
    mmp.Checkerboard() = int(src.Checkerboard());
    r.Checkerboard() = int(src.Checkerboard());
    const RealD ssq = norm2(src);
    RealD d, b, c, cp;
    Linop.HermOpAndNorm(psi, mmp, d, b);
    axpby(r, 1.0, -1.0, src, mmp);  // r = src - A psi
    p = r;
    cp = norm2(r);
    const RealD rsq = Tolerance * Tolerance * ssq;
    IterationsToComplete = 0;
    if (cp <= rsq) {
      TrueResidual = ssq > 0 ? std::sqrt(cp / ssq) : 0;
      return;
    }
    for (int k = 1; k <= MaxIterations; k++) {
      c = cp;
      Linop.HermOpAndNorm(p, mmp, d, b);
      const RealD a = c / d;
      cp = axpy_norm(r, -a, mmp, r);
      b = cp / c;
      axpy(psi, a, p, psi);
      axpby(p, b, 1.0, p, r);
      if (cp <= rsq) {
        Linop.HermOp(psi, mmp);
        axpby(p, 1.0, -1.0, mmp, src);
        TrueResidual = std::sqrt(norm2(p) / ssq);
        IterationsToComplete = k;
        return;
      }
    }
    IterationsToComplete = MaxIterations;
    if (ErrorOnNoConverge) throw GridError(GB_ERR_NOT_CONVERGED, "ConjugateGradient did not converge");
  }
};

// ConjugateGradientReliableUpdate<FieldD, FieldF>(tol, maxit, delta, sp_grid, Linop_f,
// Linop_d, err_on_nonconv) (ConjugateGradientReliableUpdate.h:33-270): FP32 (or FP16)
// inner CG with FP64 reliable updates.  Both linear operators must be library operators
// of the same kind.
template <class FieldD, class FieldF> class ConjugateGradientReliableUpdate : public LinearFunction<FieldD> {
 public:
  RealD Tolerance, Delta;
  Integer MaxIterations;
  bool ErrorOnNoConverge, DoFinalCleanup = true;
  Integer IterationsToComplete = 0, IterationsToCleanup = 0, ReliableUpdatesPerformed = 0;
  RealD TrueResidual = 0;
  Integer ReliableUpdateEvery = 100;  // also update at least this often (0 = only on Delta)
  bool UseGraphs = false;
  LinearOperatorBase<FieldF>& Linop_f;
  LinearOperatorBase<FieldD>& Linop_d;

  ConjugateGradientReliableUpdate(RealD tol, Integer maxit, RealD delta, GridBase*, LinearOperatorBase<FieldF>& lf,
                                  LinearOperatorBase<FieldD>& ld, bool err_on_nonconv = true)
      : Tolerance(tol), Delta(delta), MaxIterations(maxit), ErrorOnNoConverge(err_on_nonconv), Linop_f(lf),
        Linop_d(ld) {}

  void operator()(const FieldD& src, FieldD& psi) override {
    gb_op_t od = Linop_d.library_op(), of = Linop_f.library_op();
    if (!od || !of || Linop_d.library_kind() != Linop_f.library_kind())
      throw GridError(GB_ERR_UNSUPPORTED, "ConjugateGradientReliableUpdate: library operators of one kind expected");
    gb_cg_params p;
    gb_cg_params_default(&p);
    p.tolerance = Tolerance;
    p.max_iterations = MaxIterations;
    p.err_on_no_conv = ErrorOnNoConverge ? 1 : 0;
    p.delta = Delta;
    p.relup_every = ReliableUpdateEvery;
    p.final_cleanup = DoFinalCleanup ? 1 : 0;
    p.use_graphs = UseGraphs ? 1 : 0;
    gb_cg_result r;
    const int rc = gb_cg_reliable(od, of, Linop_d.library_kind(), src.handle(), psi.handle(), &p, &r);
    IterationsToComplete = r.iterations;
    IterationsToCleanup = r.cleanup_iterations;
    ReliableUpdatesPerformed = r.reliable_updates;
    TrueResidual = r.true_residual;
    gbdetail::check(rc, "ConjugateGradientReliableUpdate");
  }
};

// MixedPrecisionConjugateGradient (ConjugateGradientMixedPrec.h:34-166): restarted FP32
// inner CGs with FP64 outer residuals and a final FP64 patch-up CG.  Errors throw
// (Grid asserts); the patch-up honours ErrorOnNoConverge of Grid's inner solvers (off).
template <class FieldD, class FieldF> class MixedPrecisionConjugateGradient : public LinearFunction<FieldD> {
 public:
  RealD Tolerance, InnerTolerance;
  Integer MaxInnerIterations, MaxOuterIterations, MaxPatchupIterations = 0;
  RealD OuterLoopNormMult = 100.;
  Integer TotalInnerIterations = 0, TotalOuterIterations = 0, TotalFinalStepIterations = 0;
  RealD TrueResidual = 0;
  bool UseGraphs = false;
  LinearOperatorBase<FieldF>& Linop_f;
  LinearOperatorBase<FieldD>& Linop_d;

  MixedPrecisionConjugateGradient(RealD tol, Integer maxinnerit, Integer maxouterit, GridBase*,
                                  LinearOperatorBase<FieldF>& lf, LinearOperatorBase<FieldD>& ld)
      : Tolerance(tol), InnerTolerance(tol), MaxInnerIterations(maxinnerit), MaxOuterIterations(maxouterit),
        Linop_f(lf), Linop_d(ld) {}

  void operator()(const FieldD& src, FieldD& psi) override {
    gb_op_t od = Linop_d.library_op(), of = Linop_f.library_op();
    if (!od || !of || Linop_d.library_kind() != Linop_f.library_kind())
      throw GridError(GB_ERR_UNSUPPORTED, "MixedPrecisionConjugateGradient: library operators of one kind expected");
    gb_cg_params p;
    gb_cg_params_default(&p);
    p.tolerance = Tolerance;
    p.err_on_no_conv = 0;
    p.use_graphs = UseGraphs ? 1 : 0;
    gb_mixed_params m;
    gb_mixed_params_default(&m);
    m.inner_tolerance = InnerTolerance;
    m.max_inner_iterations = MaxInnerIterations;
    m.max_outer_iterations = MaxOuterIterations;
    m.max_patchup_iterations = MaxPatchupIterations;
    m.outer_loop_norm_mult = OuterLoopNormMult;
    gb_cg_result r;
    const int rc = gb_cg_mixed(od, of, Linop_d.library_kind(), src.handle(), psi.handle(), &p, &m, &r);
    TotalInnerIterations = r.iterations;
    TotalOuterIterations = r.reliable_updates;
    TotalFinalStepIterations = r.cleanup_iterations;
    TrueResidual = r.true_residual;
    gbdetail::check(rc, "MixedPrecisionConjugateGradient");
  }
};

// MixedPrecisionConjugateGradientBatched (ConjugateGradientMixedPrecBatched.h:37-209):
// the right-hand sides of a multi-RHS operator pair are solved together by the solver
// above; the vector form solves them one after the other, as Grid's does
template <class FieldD, class FieldF> class MixedPrecisionConjugateGradientBatched
    : public MixedPrecisionConjugateGradient<FieldD, FieldF> {
  typedef MixedPrecisionConjugateGradient<FieldD, FieldF> Base;

 public:
  MixedPrecisionConjugateGradientBatched(RealD tol, Integer maxinnerit, Integer maxouterit, Integer maxpatchit,
                                         GridBase* g, LinearOperatorBase<FieldF>& lf, LinearOperatorBase<FieldD>& ld,
                                         bool = true)
      : Base(tol, maxinnerit, maxouterit, g, lf, ld) {
    this->MaxPatchupIterations = maxpatchit;
  }
  using Base::operator();
  void operator()(const std::vector<FieldD>& src, std::vector<FieldD>& sol) {
    if (src.size() != sol.size()) throw GridError(GB_ERR_BAD_ARG, "MixedPrecisionConjugateGradientBatched: sizes differ");
    for (size_t i = 0; i < src.size(); i++) Base::operator()(src[i], sol[i]);
  }
};

// MultiShiftFunction (Grid/algorithms/approx/MultiShiftFunction.h:34-64): a partial-fraction
// rational function f(x) = norm + sum_i residues[i] / (x + poles[i]).  The Remez
// construction of Grid's AlgRemez is not part of this library: fill the arrays directly.
class MultiShiftFunction {
 public:
  int order = 0;
  std::vector<RealD> poles, residues, tolerances;
  RealD norm = 0, lo = 0, hi = 0;
  MultiShiftFunction() {}
  MultiShiftFunction(int n, RealD _lo, RealD _hi) : order(n), poles(n), residues(n), tolerances(n), lo(_lo), hi(_hi) {}
  RealD approx(RealD x) const {
    RealD a = norm;
    for (int i = 0; i < order; i++) a += residues[i] / (x + poles[i]);
    return a;
  }
};

// ConjugateGradientMultiShift(maxit, shifts) (ConjugateGradientMultiShift.h:44-75): solves
// (A + poles[i]) results[i] = src for every pole at once on a library linear operator;
// the one-field form returns norm src + sum_i residues[i] results[i].
template <class Field> class ConjugateGradientMultiShift : public OperatorFunction<Field> {
 public:
  Integer MaxIterations;
  Integer IterationsToComplete = 0;
  std::vector<int> IterationsToCompleteShift;
  std::vector<RealD> TrueResidualShift;
  MultiShiftFunction shifts;
  int CheckEvery = 10;
  ConjugateGradientMultiShift(Integer maxit, const MultiShiftFunction& s)
      : MaxIterations(maxit), IterationsToCompleteShift(s.order), TrueResidualShift(s.order), shifts(s) {}

  void operator()(LinearOperatorBase<Field>& Linop, const Field& src, std::vector<Field>& results) {
    gb_op_t op = Linop.library_op();
    if (!op) throw GridError(GB_ERR_UNSUPPORTED, "ConjugateGradientMultiShift: a library linear operator expected");
    if (int(results.size()) != shifts.order) throw GridError(GB_ERR_BAD_ARG, "one result field per pole expected");
    std::vector<gb_field_t> h(results.size());
    for (size_t i = 0; i < results.size(); i++) h[i] = results[i].handle();
    gb_multishift_result r;
    const int rc = gb_cg_multishift(op, Linop.library_kind(), src.handle(), shifts.order, shifts.poles.data(),
                                    shifts.tolerances.data(), h.data(), MaxIterations, CheckEvery, &r);
    IterationsToComplete = r.iterations;
    for (int i = 0; i < shifts.order; i++) {
      IterationsToCompleteShift[i] = r.iterations_shift[i];
      TrueResidualShift[i] = r.true_residual_shift[i];
    }
    gbdetail::check(rc, "ConjugateGradientMultiShift");
  }
  void operator()(LinearOperatorBase<Field>& Linop, const Field& src, std::vector<Field>& results, Field& psi) {
    (*this)(Linop, src, results);
    axpby(psi, shifts.norm, 0.0, src, src);
    for (int i = 0; i < shifts.order; i++) axpby(psi, 1.0, shifts.residues[i], psi, results[i]);
  }
  void operator()(LinearOperatorBase<Field>& Linop, const Field& src, Field& psi) override {
    std::vector<Field> results;
    results.reserve(shifts.order);
    for (int i = 0; i < shifts.order; i++) {
      results.emplace_back(src.Grid());
      results.back().Checkerboard() = int(src.Checkerboard());
    }
    (*this)(Linop, src, results, psi);
  }
};

// SchurRedBlackDiagMooeeSolve(OperatorFunction&) (SchurRedBlack.h:373-436).  The CG is a
// library ConjugateGradient; an optional lower-precision operator of the same action
// turns the inner solve into the mixed-precision reliable-update CG.
template <class Field> class SchurRedBlackDiagMooeeSolve {
  OperatorFunction<Field>& solver_;

 public:
  Integer IterationsToComplete = 0;
  RealD TrueResidual = 0, UnpreconditionedResidual = 0;
  explicit SchurRedBlackDiagMooeeSolve(OperatorFunction<Field>& HermitianRBSolver, bool = false, bool = false)
      : solver_(HermitianRBSolver) {}
  template <class Matrix> void operator()(Matrix& _Matrix, const Field& in, Field& out) { solve(_Matrix, nullptr, in, out); }
  // with an initial-guess functor (SchurRedBlack.h:189-233); the library solve starts from
  // zero, so only ZeroGuesser is accepted
  template <class Matrix, class Guesser, typename std::enable_if<Guesser::is_zero_guesser, int>::type = 0>
  void operator()(Matrix& _Matrix, const Field& in, Field& out, Guesser&) {
    solve(_Matrix, nullptr, in, out);
  }
  template <class Matrix, class MatrixLo>
  void operator()(Matrix& _Matrix, MatrixLo& lower_precision, const Field& in, Field& out) {
    solve(_Matrix, lower_precision.handle(), in, out);
  }
  // the gb_cg_solver of the library's solver functions (gb_solver_pv_rbprec, ...) for this
  // solver, and the results of such a call taken back
  gb_cg_solver solver_state(gb_op_t lo = nullptr) const {
    gb_cg_solver st{};
    st.cg = cg().params();
    st.op_lo = lo;
    return st;
  }
  void take_result(const gb_cg_solver& st) {
    IterationsToComplete = cg().IterationsToComplete = st.result.iterations;
    TrueResidual = cg().TrueResidual = st.result.true_residual;
  }

 private:
  ConjugateGradient<Field>& cg() const {
    auto* cg = dynamic_cast<ConjugateGradient<Field>*>(&solver_);
    if (!cg) throw GridError(GB_ERR_UNSUPPORTED, "SchurRedBlackDiagMooeeSolve: a ConjugateGradient solver expected");
    return *cg;
  }
  template <class Matrix> void solve(Matrix& M, gb_op_t lo, const Field& in, Field& out) {
    ConjugateGradient<Field>* cg = &this->cg();
    const gb_cg_params p = cg->params();
    gb_cg_result r;
    // one unpreconditioned residual per right-hand side (slot) of the operator
    int ls = 0, nrhs = 1, prec = 0;
    int64_t half4 = 0;
    gbdetail::check(gb_op_info(M.handle(), &ls, &nrhs, &half4, &prec), "SchurRedBlackDiagMooeeSolve");
    std::vector<double> unprec_v(size_t(nrhs > 0 ? nrhs : 1), 0.0);
    const int rc = gb_schur_solve(M.handle(), lo, in.handle(), out.handle(), &p, &r, unprec_v.data());
    double unprec = 0;
    for (double v : unprec_v) unprec = std::max(unprec, v);
    IterationsToComplete = cg->IterationsToComplete = r.iterations;
    TrueResidual = cg->TrueResidual = r.true_residual;
    UnpreconditionedResidual = unprec;
    gbdetail::check(rc, "SchurRedBlackDiagMooeeSolve");
  }
};

// ---- MADWF (Grid/qcd/action/fermion/MADWF.h, PauliVillarsInverters.h) ----------------
// ZeroGuesser (Grid/algorithms/iterative/Guesser.h)
template <class Field> struct ZeroGuesser {
  static constexpr bool is_zero_guesser = true;
  void operator()(const Field&, Field& guess) { guess = Zero(); }
};

// PauliVillarsSolverUnprec (PauliVillarsInverters.h:32-52): M(1) sol = src by CG on Mdag M
// (the library's gb_solver_pv_unprec, which restores the mass)
template <class Field> class PauliVillarsSolverUnprec {
 public:
  ConjugateGradient<Field>& CG;
  explicit PauliVillarsSolverUnprec(ConjugateGradient<Field>& cg) : CG(cg) {}
  template <class Matrix> void operator()(Matrix& _Matrix, const Field& src, Field& sol) {
    gb_cg_solver st{};
    st.cg = CG.params();
    const int rc = gb_solver_pv_unprec(&st, _Matrix.handle(), src.handle(), sol.handle());
    CG.IterationsToComplete = st.result.iterations;
    CG.TrueResidual = st.result.true_residual;
    gbdetail::check(rc, "PauliVillarsSolverUnprec");
  }
};

// PauliVillarsSolverRBprec (PauliVillarsInverters.h:54-72): the Schur solve at mass 1 (the
// library's gb_solver_pv_rbprec); SchurSolverType provides solver_state / take_result
template <class Field, class SchurSolverType> class PauliVillarsSolverRBprec {
 public:
  SchurSolverType& SchurSolver;
  explicit PauliVillarsSolverRBprec(SchurSolverType& s) : SchurSolver(s) {}
  template <class Matrix> void operator()(Matrix& _Matrix, const Field& src, Field& sol) {
    gb_cg_solver st = SchurSolver.solver_state();
    const int rc = gb_solver_pv_rbprec(&st, _Matrix.handle(), src.handle(), sol.handle());
    SchurSolver.take_result(st);
    gbdetail::check(rc, "PauliVillarsSolverRBprec");
  }
};

namespace gbdetail {
// gb_pv_fourier_t owned by an adapter object
class PVFourier {
  gb_pv_fourier_t h_ = nullptr;

 public:
  PVFourier(const double* U, const gb_cg_params& p, int group_in_s) {
    check(gb_pv_fourier_create(U, &p, group_in_s, &h_), "FourierAcceleratedPV");
  }
  PVFourier(const PVFourier&) = delete;
  PVFourier& operator=(const PVFourier&) = delete;
  ~PVFourier() { gb_pv_fourier_destroy(h_); }
  template <class Field> void solve(gb_op_t op, ConjugateGradient<Field>& cg, const Field& src, Field& dst) const {
    const gb_cg_params p = cg.params();
    check(gb_pv_fourier_set_params(h_, &p), "FourierAcceleratedPV");
    const int rc = gb_solver_pv_fourier(h_, op, src.handle(), dst.handle());
    gb_cg_result r{};
    gb_pv_fourier_result(h_, &r);
    cg.IterationsToComplete = r.iterations;
    cg.TrueResidual = r.true_residual;
    check(rc, "FourierAcceleratedPV");
  }
};
}  // namespace gbdetail

// FourierAcceleratedPV (FourierAcceleratedPV.h:56-237): the Pauli-Villars (mass 1) inverse of
// a Moebius operator with constant real b, c by the library's gb_solver_pv_fourier: a
// twisted DFT along s block-diagonalises it, modes s and Ls-1-s pair into 5D twisted-mass
// Wilson systems (group_in_s pairs at a time) solved by the red-black Schur CG, and the
// recombined solutions are transformed back.  Umu must outlive the object.
template <class Field, class Matrix, class GaugeField> class FourierAcceleratedPV {
  Matrix& dwfPV;
  ConjugateGradient<Field>& cg;
  gbdetail::PVFourier pv_;

 public:
  FourierAcceleratedPV(Matrix& m, const GaugeField& U, ConjugateGradient<Field>& c, int g = 2)
      : dwfPV(m), cg(c), pv_(reinterpret_cast<const double*>(U.data.data()), c.params(), g) {
    if (dwfPV.Ls % (2 * g) != 0) throw GridError(GB_ERR_BAD_ARG, "FourierAcceleratedPV: Ls % (2 group_in_s)");
  }
  void pvInv(const Field& src, Field& dst) const { pv_.solve(dwfPV.handle(), cg, src, dst); }
};

// PauliVillarsSolverFourierAccel (PauliVillarsInverters.h:74-88); the library keeps its
// twisted-mass operator from one call to the next
template <class Field, class GaugeField> class PauliVillarsSolverFourierAccel {
  gbdetail::PVFourier pv_;

 public:
  const GaugeField& Umu;
  ConjugateGradient<Field>& CG;
  PauliVillarsSolverFourierAccel(const GaugeField& U, ConjugateGradient<Field>& cg)
      : pv_(reinterpret_cast<const double*>(U.data.data()), cg.params(), 2), Umu(U), CG(cg) {}
  template <class Matrix> void operator()(Matrix& _Matrix, const Field& src, Field& sol) {
    pv_.solve(_Matrix.handle(), CG, src, sol);
  }
};

struct MADWFinnerIterCallbackBase {
  virtual void operator()(const RealD) {}
  virtual ~MADWFinnerIterCallbackBase() {}
};

// MADWF (MADWF.h:47-209): the library's gb_madwf solves the outer (Moebius) system by
// defect correction, each step a Pauli-Villars solve of the outer operator and a Schur
// solve of the cheaper inner one, joined through the s = 0 slice of the P-rotated fields;
// the solver objects, the guesser and the callback are called back from it.  src is a 4D
// field (imported with ImportPhysicalFermionSource) or a 5D field of the outer operator.
// Throws GridError (GB_ERR_NOT_CONVERGED) after maxiter steps, where Grid asserts; an
// exception from a solver or the callback ends the solve and is rethrown.
template <class Matrixo, class Matrixi, class PVinverter, class SchurSolver, class Guesser> class MADWF {
  typedef typename Matrixo::FermionField FermionFieldo;
  typedef typename Matrixi::FermionField FermionFieldi;
  Matrixo& Mato;
  Matrixi& Mati;
  PVinverter& PauliVillarsSolvero;
  SchurSolver& SchurSolveri;
  Guesser& Guesseri;
  RealD target_resid;
  int maxiter;
  MADWFinnerIterCallbackBase* callback;
  std::exception_ptr error_;

  template <class Body> int guarded(Body&& body) {
    try {
      body();
      return GB_OK;
    } catch (const GridError& e) {
      if (!error_) error_ = std::current_exception();
      return e.status != GB_OK ? e.status : GB_ERR_BAD_ARG;
    } catch (...) {
      if (!error_) error_ = std::current_exception();
      return GB_ERR_BAD_ARG;
    }
  }
  static int pv_call(void* user, gb_op_t, gb_field_t src, gb_field_t sol) {
    MADWF* m = static_cast<MADWF*>(user);
    return m->guarded([&] {
      const FermionFieldo s = FermionFieldo::View(m->Mato.FermionGrid(), src);
      FermionFieldo x = FermionFieldo::View(m->Mato.FermionGrid(), sol);
      m->PauliVillarsSolvero(m->Mato, s, x);
    });
  }
  static int inner_call(void* user, gb_op_t, gb_field_t src, gb_field_t sol) {
    MADWF* m = static_cast<MADWF*>(user);
    return m->guarded([&] {
      const FermionFieldi s = FermionFieldi::View(m->Mati.FermionGrid(), src);
      FermionFieldi x = FermionFieldi::View(m->Mati.FermionGrid(), sol);
      m->SchurSolveri(m->Mati, s, x, m->Guesseri);
    });
  }
  static int step_call(void* user, int, double resid) {
    MADWF* m = static_cast<MADWF*>(user);
    return m->guarded([&] {
      if (m->callback) (*m->callback)(resid);
    });
  }

 public:
  int IterationsToComplete = 0;
  RealD FinalResidual = 0;
  MADWF(Matrixo& _Mato, Matrixi& _Mati, PVinverter& _PV, SchurSolver& _SchurSolveri, Guesser& _Guesseri, RealD resid,
        int _maxiter, MADWFinnerIterCallbackBase* _callback = nullptr)
      : Mato(_Mato), Mati(_Mati), PauliVillarsSolvero(_PV), SchurSolveri(_SchurSolveri), Guesseri(_Guesseri),
        target_resid(resid), maxiter(_maxiter), callback(_callback) {}

  void operator()(const FermionFieldo& src, FermionFieldo& sol5) {
    std::unique_ptr<FermionFieldo> b;
    gb_field_t src5 = src.handle();
    if (src.Grid() == Mato.GaugeGrid()) {
      b.reset(new FermionFieldo(Mato.FermionGrid()));
      Mato.ImportPhysicalFermionSource(src, *b);
      src5 = b->handle();
    } else if (src.Grid() != Mato.FermionGrid()) {
      throw GridError(GB_ERR_BAD_ARG, "MADWF: source on neither the gauge nor the fermion grid of the outer operator");
    }
    error_ = nullptr;
    int it = 0;
    double fr = 0;
    const int rc = gb_madwf(Mato.handle(), Mati.handle(), &MADWF::pv_call, this, &MADWF::inner_call, this, src5,
                            sol5.handle(), target_resid, maxiter, &MADWF::step_call, this, &it, &fr);
    IterationsToComplete = it;
    FinalResidual = fr;
    if (error_) std::rethrow_exception(error_);
    if (rc == GB_ERR_NOT_CONVERGED) throw GridError(GB_ERR_NOT_CONVERGED, "MADWF: exceeded maxiter");
    gbdetail::check(rc, "MADWF");
  }
};

}  // namespace Grid

#endif  // GBGRID_H
