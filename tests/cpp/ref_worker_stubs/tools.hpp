// Stand-in for the reference's src/tools.hpp as gpuWorker.cpp uses it: the
// debug-level flags and a stream-style debug writer that prints only when
// the level is enabled. TEST INFRASTRUCTURE ONLY.
#pragma once
#include <iostream>
#include <sstream>
#include <string>

enum debugLevel : unsigned char { cpu = 1, gpu = 1 << 1, net = 1 << 2, info = 1 << 3,
                                  parameter = 1 << 4, kernel = 1 << 5 };

class AtomicWriter {
  public:
    AtomicWriter(unsigned char enabled, debugLevel level) : on_((enabled & level) != 0) {}
    template <typename T> AtomicWriter &operator<<(const T &x) {
        if (on_) buf_ << x;
        return *this;
    }
    ~AtomicWriter() {
        if (on_) std::cout << buf_.str();
    }

  private:
    bool on_;
    std::ostringstream buf_;
};
