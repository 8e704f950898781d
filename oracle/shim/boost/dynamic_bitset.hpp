// Minimal stand-in for boost::dynamic_bitset<> covering what the sDbscan
// reference sources use (ctor(n), operator[] read/assign, count, clear,
// find_first, find_next, npos).  Written from scratch for the oracle build:
// Boost is not installed on this machine.  Test infrastructure only.
//
// One deliberate difference: setting a bit is an atomic OR on its word.  The
// reference sets core flags from inside `#pragma omp parallel for`
// (src/sDbscan.cpp:384, :1436), which with a plain bitset is a data race on
// shared words; the atomic form gives the race-free result the code intends.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace boost {

template <typename Block = unsigned long> class dynamic_bitset {
    std::vector<Block> w_;
    std::size_t n_ = 0;
    static const std::size_t B = sizeof(Block) * 8;

public:
    static const std::size_t npos = static_cast<std::size_t>(-1);

    class reference {
        Block* word_;
        Block mask_;

    public:
        reference(Block* w, Block m) : word_(w), mask_(m) {}
        operator bool() const { return (__atomic_load_n(word_, __ATOMIC_RELAXED) & mask_) != 0; }
        bool operator!() const { return !static_cast<bool>(*this); }
        reference& operator=(bool v) {
            if (v) __atomic_fetch_or(word_, mask_, __ATOMIC_RELAXED);
            else __atomic_fetch_and(word_, ~mask_, __ATOMIC_RELAXED);
            return *this;
        }
        reference& operator=(const reference& o) { return *this = static_cast<bool>(o); }
    };

    dynamic_bitset() {}
    explicit dynamic_bitset(std::size_t n) : w_((n + B - 1) / B, Block(0)), n_(n) {}

    std::size_t size() const { return n_; }
    reference operator[](std::size_t i) { return reference(&w_[i / B], Block(1) << (i % B)); }
    bool operator[](std::size_t i) const { return (w_[i / B] >> (i % B)) & 1; }
    bool test(std::size_t i) const { return (*this)[i]; }

    std::size_t count() const {
        std::size_t c = 0;
        for (Block b : w_) c += static_cast<std::size_t>(__builtin_popcountll(static_cast<unsigned long long>(b)));
        return c;
    }
    void clear() {
        w_.clear();
        n_ = 0;
    }
    std::size_t find_from(std::size_t i) const {
        if (i >= n_) return npos;
        std::size_t wi = i / B;
        Block b = w_[wi] & (~Block(0) << (i % B));
        while (true) {
            if (b) {
                std::size_t pos = wi * B + static_cast<std::size_t>(__builtin_ctzll(static_cast<unsigned long long>(b)));
                return pos < n_ ? pos : npos;
            }
            if (++wi >= w_.size()) return npos;
            b = w_[wi];
        }
    }
    std::size_t find_first() const { return find_from(0); }
    std::size_t find_next(std::size_t pos) const { return pos + 1 >= n_ ? npos : find_from(pos + 1); }
};

}  // namespace boost
