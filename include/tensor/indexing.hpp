// Labelled index iteration (the reference's TIndexing, include/tensor/indexing.hpp:9-166).
// Host-side; the device kernels use stride arithmetic instead. Iteration order: indices
// are visited fastest-first in descending tag order, and among equal tags the last index
// is fastest.
#ifndef QTNH_TENSOR_INDEXING_HPP
#define QTNH_TENSOR_INDEXING_HPP

#include <ostream>
#include <string>
#include <vector>

#include "core/typedefs.hpp"

namespace qtnh {
  struct TIFlag {
    std::string label;
    int tag;

    bool operator==(const TIFlag& rhs) const { return label == rhs.label && tag == rhs.tag; }
    bool operator!=(const TIFlag& rhs) const { return !(*this == rhs); }

    TIFlag() : TIFlag("default", 0) {}
    TIFlag(std::string label, int tag) : label(label), tag(tag) {}
  };

  namespace ops {
    std::ostream& operator<<(std::ostream&, const qtnh::tidx_tup&);
    std::ostream& operator<<(std::ostream&, const TIFlag&);
  }

  class TIndexing {
    public:
      TIndexing(qtnh::tidx_tup dims);
      TIndexing(qtnh::tidx_tup dims, std::vector<TIFlag> ifls);

      const qtnh::tidx_tup& dims() const noexcept { return dims_; }
      const std::vector<TIFlag>& ifls() const noexcept { return ifls_; }

      bool isValid(qtnh::tidx_tup idxs) const;
      bool isEqual(qtnh::tidx_tup idxs1, qtnh::tidx_tup idxs2, std::string ifl_label = "default") const;
      bool isLast(qtnh::tidx_tup idxs, std::string ifl_label = "default") const;

      /// Next tuple, advancing only indices labelled ifl_label; std::out_of_range past the end.
      qtnh::tidx_tup next(qtnh::tidx_tup idxs, std::string ifl_label = "default") const;
      /// Previous tuple; std::out_of_range before the start.
      qtnh::tidx_tup prev(qtnh::tidx_tup idxs, std::string ifl_label = "default") const;
      qtnh::tidx_tup reset(qtnh::tidx_tup idxs, std::string ifl_label = "default") const;

      TIndexing cut(std::string ifl_label = "default") const;
      TIndexing keep(std::string ifl_label = "default") const;

      struct TupIterator {
        TupIterator(qtnh::tidx_tup dims, std::vector<std::size_t> order, qtnh::tidx_tup start, bool is_end);
        TupIterator begin();
        TupIterator end();
        TupIterator& operator++();
        TupIterator operator++(int);
        bool operator!=(const TupIterator& rhs) const { return is_end_ != rhs.is_end_; }
        qtnh::tidx_tup operator*() const { return current_; }

       private:
        qtnh::tidx_tup dims_;
        std::vector<std::size_t> order_;
        qtnh::tidx_tup current_;
        bool is_end_;
      };

      struct NumIterator {
        NumIterator(qtnh::tidx_tup dims, std::vector<std::size_t> incrs, std::size_t zero, qtnh::tidx_tup current_idxs,
                    bool is_end);
        NumIterator begin();
        NumIterator end();
        NumIterator& operator++();
        NumIterator operator++(int);
        bool operator!=(const NumIterator& rhs) const { return is_end_ != rhs.is_end_; }
        std::size_t operator*() const;

       private:
        qtnh::tidx_tup dims_;
        std::vector<std::size_t> incrs_;
        std::size_t zero_;
        qtnh::tidx_tup current_idxs_;
        bool is_end_;
      };

      TupIterator tup(std::string ifl_label = "default") const;
      TupIterator tup(std::string ifl_label, qtnh::tidx_tup start) const;
      NumIterator num(std::string ifl_label = "default") const;
      NumIterator num(std::string ifl_label, qtnh::tidx_tup start) const;

      template <typename T>
      static T app(T t) {
        return t;
      }

      /// Concatenation of several indexings.
      template <typename T, typename... Args>
      static T app(T t, Args... args) {
        return _app(t, app(args...));
      }

    private:
      qtnh::tidx_tup dims_;
      std::vector<TIFlag> ifls_;
      std::vector<std::size_t> maps_;  // index positions, fastest first

      static TIndexing _app(const TIndexing& ti1, const TIndexing& ti2);
  };
}

#endif
