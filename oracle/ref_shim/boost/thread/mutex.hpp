// Minimal stand-in for boost::mutex, used only to compile the reference's
// STSC sources for the oracle. The reference includes this header from
// src/skycube/NodeAuxilliary.h:20 and needs boost::mutex with scoped_lock.
#pragma once
#include <mutex>
namespace boost {
struct mutex : std::mutex {
  struct scoped_lock {
    std::unique_lock<std::mutex> l;
    explicit scoped_lock(mutex& m) : l(m) {}
    void unlock() { l.unlock(); }
  };
};
}  // namespace boost
