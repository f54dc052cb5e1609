// Project-written stand-in for the one Boost class the reference names on its
// build path (boost::dynamic_bitset<>).  Test infrastructure only: it lets the
// oracle recipe compile the reference sources without Boost installed.
// Only the members the reference uses exist: (size, value) construction,
// operator[], reset(), size().  There is deliberately no initializer_list
// constructor, so `flags{n, 0}` means "n bits, all zero" as it does in Boost.
#pragma once
#include <cstddef>
#include <vector>
namespace boost {
template <class Block = unsigned long>
class dynamic_bitset {
 public:
  dynamic_bitset() {}
  dynamic_bitset(std::size_t n, unsigned long v) : bits_(n, false) {
    for (std::size_t i = 0; i < n && i < 8 * sizeof(unsigned long); ++i) bits_[i] = (v >> i) & 1ul;
  }
  std::vector<bool>::reference operator[](std::size_t i) { return bits_[i]; }
  bool operator[](std::size_t i) const { return bits_[i]; }
  dynamic_bitset &reset() {
    std::fill(bits_.begin(), bits_.end(), false);
    return *this;
  }
  std::size_t size() const { return bits_.size(); }

 private:
  std::vector<bool> bits_;
};
}  // namespace boost
