// TensorNetwork (src/tensor/network.cpp:1-204 of the reference): a registry of tensors
// and bonds; contracting a bond rewires the remaining bonds through the dimension
// replacements the contraction chose. Tensors stay in HBM between contractions.
#include <iostream>

#include "qtnh.hpp"

namespace qtnh {

TensorNetwork::TensorNetwork() = default;

TensorNetwork::Bond::Bond(std::pair<qtnh::uint, qtnh::uint> tids, std::vector<qtnh::wire> ws) : tensor_ids(tids), wires(ws) {}

Tensor* TensorNetwork::tensor(qtnh::uint tid) { return tensors_.at(tid).get(); }

const TensorNetwork::Bond& TensorNetwork::bond(qtnh::uint bid) { return bonds_.at(bid); }

std::vector<qtnh::uint> TensorNetwork::tensorIDs() {
  std::vector<qtnh::uint> ids;
  for (auto& kv : tensors_) ids.push_back(kv.first);
  return ids;
}

std::vector<qtnh::uint> TensorNetwork::bondIDs() {
  std::vector<qtnh::uint> ids;
  for (auto& kv : bonds_) ids.push_back(kv.first);
  return ids;
}

qtnh::tptr TensorNetwork::extract(qtnh::uint tid) {
  auto tp = std::move(tensors_.at(tid));
  tensors_.erase(tid);
  return tp;
}

qtnh::uint TensorNetwork::insert(qtnh::tptr tp) {
  tensors_.insert({++tensor_counter, std::move(tp)});
  return tensor_counter;
}

qtnh::uint TensorNetwork::addBond(qtnh::uint tid1, qtnh::uint tid2, std::vector<qtnh::wire> ws) {
  bonds_.insert({++bond_counter, Bond({tid1, tid2}, ws)});
  return bond_counter;
}

qtnh::uint TensorNetwork::contractBond(qtnh::uint bid) {
  auto& b = bonds_.at(bid);
  const auto tid1 = b.tensor_ids.first, tid2 = b.tensor_ids.second;
  ConParams params(b.wires);
  auto tp3 = Tensor::contract(std::move(tensors_.at(tid1)), std::move(tensors_.at(tid2)), params);
  const auto r1 = params.dimRepls1, r2 = params.dimRepls2;
  bonds_.erase(bid);
  tensors_.erase(tid1);
  tensors_.erase(tid2);
  const auto tid3 = insert(std::move(tp3));
  for (auto& kv : bonds_) {
    Bond& o = kv.second;
    if (o.tensor_ids.first == tid1) {
      o.tensor_ids.first = tid3;
      for (auto& w : o.wires) w.first = r1.at(w.first);
    } else if (o.tensor_ids.first == tid2) {
      o.tensor_ids.first = tid3;
      for (auto& w : o.wires) w.first = r2.at(w.first);
    }
    if (o.tensor_ids.second == tid1) {
      o.tensor_ids.second = tid3;
      for (auto& w : o.wires) w.second = r1.at(w.second);
    } else if (o.tensor_ids.second == tid2) {
      o.tensor_ids.second = tid3;
      for (auto& w : o.wires) w.second = r2.at(w.second);
    }
  }
  return tid3;
}

qtnh::uint TensorNetwork::contractAll() {
  auto tid = tensors_.begin()->first;
  auto temp = bonds_;
  for (auto& kv : temp) tid = contractBond(kv.first);
  return tid;
}

qtnh::uint TensorNetwork::contractAll(std::vector<qtnh::uint> order) {
  auto tid = tensors_.begin()->first;
  for (std::size_t i = 0, j = 1; i < order.size(); i += j) {
    const auto bid1 = order.at(i);
    auto& b1 = bonds_.at(bid1);
    for (j = 1; i + j < order.size(); ++j) {
      const auto bid2 = order.at(i + j);
      auto b2 = bonds_.at(bid2);
      if (b1.tensor_ids.first == b2.tensor_ids.first && b1.tensor_ids.second == b2.tensor_ids.second) {
        b1.wires.insert(b1.wires.end(), b2.wires.begin(), b2.wires.end());
        bonds_.erase(bid2);
      } else {
        break;
      }
    }
    tid = contractBond(bid1);
    tensors_.at(tid) = Tensor::rebcast(std::move(tensors_.at(tid)), {1, 1, 0});
  }
  return tid;
}

void TensorNetwork::print() {
  using namespace qtnh::ops;
  std::cout << "================================================================\n";
  std::cout << "Tensor Network of " << tensors_.size() << " tensors and " << bonds_.size() << " bonds\n";
  std::cout << "----------------------------------------------------------------\n";
  std::cout << "Tensors: \n";
  for (auto& kv : tensors_) std::cout << "ID: " << kv.first << " | Els: " << *kv.second << "\n";
  std::cout << "----------------------------------------------------------------\n";
  std::cout << "Bonds: \n";
  for (auto& kv : bonds_) std::cout << "ID: " << kv.first << " | Bond: " << kv.second << "\n";
  std::cout << "================================================================\n";
}

std::ostream& ops::operator<<(std::ostream& out, const TensorNetwork::Bond& o) {
  out << "(" << o.tensor_ids.first << ", " << o.tensor_ids.second << "); {";
  for (std::size_t i = 0; i < o.wires.size(); ++i) {
    out << "(" << o.wires[i].first << ", " << o.wires[i].second << ")";
    if (i + 1 < o.wires.size()) out << ", ";
  }
  return out << "}";
}

}  // namespace qtnh
