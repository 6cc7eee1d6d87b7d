/*
 * Minimal host-only stand-in for <sycl/sycl.hpp>, written for this project so
 * that the reference's solver and config sources (header-only math plus the
 * INI/params code) compile with plain g++ as a CPU oracle. Only the names those
 * files touch are provided; nothing here launches device work.
 * TEST INFRASTRUCTURE ONLY.
 */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>

namespace sycl {
using std::fabs;
using std::floor;
using std::fmod;
using std::sin;
template <class T> inline T min(T a, T b) { return a < b ? a : b; }

struct queue {};
template <class T> inline T *malloc_device(std::size_t n, queue &) {
    return static_cast<T *>(std::malloc(n * sizeof(T)));
}
template <class T, int D> struct local_accessor {};
}  // namespace sycl
