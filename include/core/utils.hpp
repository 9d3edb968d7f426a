// Helper functions of the qtnh API, with the reference's names and semantics
// (include/core/utils.hpp:9-117, src/core/utils.cpp:7-74).
#ifndef QTNH_CORE_UTILS_HPP
#define QTNH_CORE_UTILS_HPP

#include <memory>
#include <ostream>
#include <stdexcept>
#include <utility>
#include <vector>

#include "core/typedefs.hpp"

namespace qtnh {
  namespace utils {
    /// Throws std::runtime_error("Unimplemented function!").
    void throw_unimplemented();

    /// True on the root process (the only process).
    bool is_root();

    /// Waits for all outstanding device work of the calling thread's environments.
    void barrier();

    /// Number of elements of a tensor with the given dimensions.
    std::size_t dims_to_size(qtnh::tidx_tup dims);

    /// Row-major (last index fastest) position of an index tuple.
    std::size_t idxs_to_i(qtnh::tidx_tup idxs, qtnh::tidx_tup dims);

    /// Index tuple of a row-major position.
    qtnh::tidx_tup i_to_idxs(std::size_t i, qtnh::tidx_tup dims);

    /// dims1 followed by dims2.
    qtnh::tidx_tup concat_dims(qtnh::tidx_tup dims1, qtnh::tidx_tup dims2);

    /// dims split before position n.
    std::pair<qtnh::tidx_tup, qtnh::tidx_tup> split_dims(qtnh::tidx_tup dims, qtnh::tidx_tup_st n);

    /// Every wire with its ends exchanged.
    std::vector<qtnh::wire> invert_wires(std::vector<qtnh::wire> ws);

    /// |a - b| < tol.
    bool equal(qtnh::tel a, qtnh::tel b, double tol = 1E-5);

    /// Ownership hand-off: returns u if it already owns t, otherwise a new owner of t.
    template <typename T>
    std::unique_ptr<T> one_unique(std::unique_ptr<T> u, T* t) {
      if (u.get() == t) return u;
      return std::unique_ptr<T>(t);
    }

    /// Ownership hand-off across types: deletes the old object unless it is t.
    template <typename T, typename U>
    std::unique_ptr<T> one_unique(std::unique_ptr<U> u, T* t) {
      auto p = u.release();
      if (dynamic_cast<T*>(p) != t) delete p;
      return std::unique_ptr<T>(t);
    }

    template <typename T>
    std::pair<std::vector<T>, std::vector<T>> split_vec(std::vector<T> vec, std::size_t n) {
      return {std::vector<T>(vec.begin(), vec.begin() + n), std::vector<T>(vec.begin() + n, vec.end())};
    }

    /// vec_perm[ptup[i]] = vec[i].
    template <typename T>
    std::vector<T> permute_vec(std::vector<T> vec, std::vector<qtnh::tidx_tup_st> ptup) {
      auto out = vec;
      for (std::size_t i = 0; i < vec.size(); ++i) out.at(ptup.at(i)) = vec.at(i);
      return out;
    }

    namespace wirecomp {
      constexpr bool first(qtnh::wire w1, qtnh::wire w2) { return w1.first < w2.first; }
      constexpr bool second(qtnh::wire w1, qtnh::wire w2) { return w1.second < w2.second; }
    }
  }

  namespace ops {
    template <typename T, typename U>
    std::ostream& operator<<(std::ostream& out, const std::pair<T, U>& p) {
      out << "(" << p.first << ", " << p.second << ")";
      return out;
    }

    template <typename T>
    std::ostream& operator<<(std::ostream& out, const std::vector<T>& v) {
      for (std::size_t i = 0; i < v.size(); ++i) {
        out << v.at(i);
        if (i + 1 < v.size()) out << ", ";
      }
      return out;
    }
  }
}

#endif
