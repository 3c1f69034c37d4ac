// Minimal stand-in for the slice of the AMGCL (801a2fb) and Boost 1.66 API that the
// reference's CoefficientMatrix::solve (src/CoefficientMatrix.cpp:210-325 of joel-ho/BES)
// uses.  TEST INFRASTRUCTURE ONLY: it lets the reference's own CoefficientMatrix.cpp
// compile unmodified in the patched reference build, and routes the solve to the CPU
// block-preconditioned GMRES restatement in oracle/linsolve.hpp (Boost is not vendored
// with the reference, so AMGCL itself cannot be built here).
//
// Mapping of the reference's options:
//   precond.relax.type ilu0             -> block ILU(0) in natural cell order
//   any other precond.relax.type        -> block Jacobi
//   precond.coarsening.*                -> ignored (no multigrid hierarchy)
//   solver.type (gmres/fgmres/lgmres/bicgstab) -> right-preconditioned GMRES(30)
//   solver.maxiter, solver.tol          -> as in AMGCL: tol relative to |b|
//   precond.coarsening.aggr.block_size  -> the block size: 5 (3-D), or 4 (2-D: rho, rho u,
//                                          rho v, rho E), which is solved as the 5x5-block
//                                          system with a decoupled, identity spanwise-momentum
//                                          row (its right-hand side and solution stay exact
//                                          zeros, so the other four components see the
//                                          arithmetic of a 4x4-block solve)
#pragma once
#include <cstddef>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../../linsolve.hpp"

namespace boost {
using std::tie;
namespace property_tree {
class ptree {
 public:
  template <class T>
  void put(const std::string& key, const T& value) {
    values_[key] = static_cast<double>(value);
  }
  double get(const std::string& key, double dflt) const {
    auto it = values_.find(key);
    return it == values_.end() ? dflt : it->second;
  }

 private:
  std::map<std::string, double> values_;
};
}  // namespace property_tree
}  // namespace boost

namespace amgcl {
namespace runtime {
namespace coarsening {
enum type { ruge_stuben, aggregation, smoothed_aggregation, smoothed_aggr_emin };
}
namespace relaxation {
enum type { gauss_seidel, ilu0, iluk, ilut, damped_jacobi, spai0, spai1, chebyshev };
}
namespace solver {
enum type { cg, bicgstab, bicgstabl, gmres, lgmres, fgmres, idrs };
}
template <class Backend>
struct amg {};
template <class Backend>
struct iterative_solver {};
}  // namespace runtime

namespace backend {
template <class T>
struct builtin {};
}  // namespace backend

namespace adapter {
struct CrsView {
  std::ptrdiff_t n;
  const std::ptrdiff_t* ptr;
  const std::ptrdiff_t* col;
  const double* val;
};
inline CrsView zero_copy(std::ptrdiff_t n, const std::ptrdiff_t* ptr, const std::ptrdiff_t* col,
                         const double* val) {
  return CrsView{n, ptr, col, val};
}
}  // namespace adapter

template <class Precond, class Solver>
class make_solver {
 public:
  make_solver(const adapter::CrsView& A, const boost::property_tree::ptree& prm) {
    restart_ = 30;
    maxiter_ = static_cast<int>(prm.get("solver.maxiter", 100));
    tol_ = prm.get("solver.tol", 1e-8);
    const int relax = static_cast<int>(prm.get("precond.relax.type", runtime::relaxation::spai0));
    bs_ = static_cast<int>(prm.get("precond.coarsening.aggr.block_size", besla::NB));
    // component r of a bs x bs block -> component of the 5x5 block
    for (int r = 0; r < besla::NB; ++r) map_[r] = (bs_ == besla::NB || r < 3) ? r : 4;
    // Scalar CSR with bs x bs blocks: block row i spans scalar rows bs i..bs i + bs - 1; each
    // scalar row lists its columns in groups of bs consecutive ids (diagonal block first).
    const std::ptrdiff_t nb = A.n / bs_;
    bm_.n = nb;
    bm_.row.assign(nb + 1, 0);
    for (std::ptrdiff_t i = 0; i < nb; ++i) {
      const std::ptrdiff_t r0 = i * bs_;
      const std::ptrdiff_t len = A.ptr[r0 + 1] - A.ptr[r0];
      bm_.row[i + 1] = bm_.row[i] + len / bs_;
    }
    bm_.col.assign(bm_.row[nb], 0);
    bm_.val.assign(bm_.row[nb] * besla::NB2, 0.0);
    bm_.diag.assign(nb, -1);
    for (std::ptrdiff_t i = 0; i < nb; ++i) {
      for (int r = 0; r < bs_; ++r) {
        const std::ptrdiff_t sr = i * bs_ + r;
        std::ptrdiff_t kb = bm_.row[i];
        for (std::ptrdiff_t k = A.ptr[sr]; k < A.ptr[sr + 1]; k += bs_, ++kb) {
          const std::ptrdiff_t c = A.col[k] / bs_;
          bm_.col[kb] = c;
          if (c == i) bm_.diag[i] = kb;
          for (int q = 0; q < bs_; ++q)
            bm_.val[kb * besla::NB2 + map_[r] * besla::NB + map_[A.col[k + q] % bs_]] =
                A.val[k + q];
        }
      }
      if (bs_ != besla::NB && bm_.diag[i] >= 0)
        bm_.val[bm_.diag[i] * besla::NB2 + 3 * besla::NB + 3] = 1.0;  // decoupled row
    }
    if (relax == runtime::relaxation::ilu0) {
      std::vector<int64_t> order(nb);
      for (std::ptrdiff_t i = 0; i < nb; ++i) order[i] = i;
      pc_.setup_ilu0(bm_, order);
    } else {
      pc_.setup_jacobi(bm_);
    }
  }

  std::tuple<std::size_t, double> operator()(const std::vector<double>& b,
                                             std::vector<double>& x) const {
    if (bs_ == besla::NB) {
      besla::GmresResult r = besla::gmres(bm_, pc_, b.data(), x.data(), restart_, maxiter_, tol_);
      return std::make_tuple(static_cast<std::size_t>(r.iterations), r.rel_residual);
    }
    const std::ptrdiff_t nb = bm_.n;
    std::vector<double> b5(nb * besla::NB, 0.0), x5(nb * besla::NB, 0.0);
    for (std::ptrdiff_t i = 0; i < nb; ++i)
      for (int r = 0; r < bs_; ++r) {
        b5[i * besla::NB + map_[r]] = b[i * bs_ + r];
        x5[i * besla::NB + map_[r]] = x[i * bs_ + r];
      }
    besla::GmresResult r = besla::gmres(bm_, pc_, b5.data(), x5.data(), restart_, maxiter_, tol_);
    for (std::ptrdiff_t i = 0; i < nb; ++i)
      for (int q = 0; q < bs_; ++q) x[i * bs_ + q] = x5[i * besla::NB + map_[q]];
    return std::make_tuple(static_cast<std::size_t>(r.iterations), r.rel_residual);
  }

 private:
  besla::BlockCsr bm_;
  besla::Preconditioner pc_;
  int restart_;
  int maxiter_;
  double tol_;
  int bs_ = besla::NB;
  int map_[besla::NB] = {0, 1, 2, 3, 4};
};

}  // namespace amgcl
