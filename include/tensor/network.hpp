// Tensor networks (mirrors the reference's include/tensor/network.hpp:16-110 and
// src/tensor/network.cpp). Tensors stay in HBM between contractions.
#ifndef QTNH_TENSOR_NETWORK_HPP
#define QTNH_TENSOR_NETWORK_HPP

#include <memory>
#include <unordered_map>

#include "core/typedefs.hpp"
#include "tensor/dense.hpp"
#include "tensor/diag.hpp"
#include "tensor/symm.hpp"
#include "tensor/tensor.hpp"

namespace qtnh {
  class TensorNetwork {
    public:
      TensorNetwork();
      TensorNetwork(const TensorNetwork&) = delete;
      ~TensorNetwork() = default;

      /// Wires between two tensors of the network.
      struct Bond {
        std::pair<qtnh::uint, qtnh::uint> tensor_ids;
        std::vector<qtnh::wire> wires;

        Bond(std::pair<qtnh::uint, qtnh::uint> tids, std::vector<qtnh::wire> ws);
        ~Bond() = default;
      };

      Tensor* tensor(qtnh::uint tid);
      const Bond& bond(qtnh::uint bid);
      std::vector<qtnh::uint> tensorIDs();
      std::vector<qtnh::uint> bondIDs();

      qtnh::tptr extract(qtnh::uint tid);
      qtnh::uint insert(qtnh::tptr tp);

      template <class T, class... U>
      qtnh::uint make(U&&... us) {
        tensors_.insert({++tensor_counter, T::make(std::forward<U>(us)...)});
        return tensor_counter;
      }

      qtnh::uint addBond(qtnh::uint tid1, qtnh::uint tid2, std::vector<qtnh::wire> ws);

      /// Contracts one bond; the other bonds of both tensors are rewired through the
      /// dimension replacements. Returns the ID of the result.
      qtnh::uint contractBond(qtnh::uint bid);
      /// Contracts every bond in the map's iteration order (as the reference).
      qtnh::uint contractAll();
      /// Contracts bonds in the given order; consecutive bonds between the same pair of
      /// tensors are merged into one contraction.
      qtnh::uint contractAll(std::vector<qtnh::uint> bids);

      void print();

    private:
      // Process-wide counters, as in the reference (network.hpp:97-98).
      inline static qtnh::uint tensor_counter = 0;
      inline static qtnh::uint bond_counter = 0;

      std::unordered_map<qtnh::uint, qtnh::tptr> tensors_;
      std::unordered_map<qtnh::uint, Bond> bonds_;
  };

  namespace ops {
    std::ostream& operator<<(std::ostream&, const TensorNetwork::Bond&);
  }
}

#endif
