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
    // Scalar CSR with 5x5 blocks: block row i spans scalar rows 5i..5i+4; each scalar row
    // lists its columns in groups of 5 consecutive ids (diagonal block first).
    const std::ptrdiff_t nb = A.n / besla::NB;
    bm_.n = nb;
    bm_.row.assign(nb + 1, 0);
    for (std::ptrdiff_t i = 0; i < nb; ++i) {
      const std::ptrdiff_t r0 = i * besla::NB;
      const std::ptrdiff_t len = A.ptr[r0 + 1] - A.ptr[r0];
      bm_.row[i + 1] = bm_.row[i] + len / besla::NB;
    }
    bm_.col.assign(bm_.row[nb], 0);
    bm_.val.assign(bm_.row[nb] * besla::NB2, 0.0);
    bm_.diag.assign(nb, -1);
    for (std::ptrdiff_t i = 0; i < nb; ++i) {
      for (int r = 0; r < besla::NB; ++r) {
        const std::ptrdiff_t sr = i * besla::NB + r;
        std::ptrdiff_t kb = bm_.row[i];
        for (std::ptrdiff_t k = A.ptr[sr]; k < A.ptr[sr + 1]; k += besla::NB, ++kb) {
          const std::ptrdiff_t c = A.col[k] / besla::NB;
          bm_.col[kb] = c;
          if (c == i) bm_.diag[i] = kb;
          for (int q = 0; q < besla::NB; ++q)
            bm_.val[kb * besla::NB2 + r * besla::NB + (A.col[k + q] % besla::NB)] = A.val[k + q];
        }
      }
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
    besla::GmresResult r = besla::gmres(bm_, pc_, b.data(), x.data(), restart_, maxiter_, tol_);
    return std::make_tuple(static_cast<std::size_t>(r.iterations), r.rel_residual);
  }

 private:
  besla::BlockCsr bm_;
  besla::Preconditioner pc_;
  int restart_;
  int maxiter_;
  double tol_;
};

}  // namespace amgcl
