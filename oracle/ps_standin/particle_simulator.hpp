// Minimal stand-in for the FDPS names that the reference's hot-path headers use.
//
// TEST INFRASTRUCTURE ONLY. This header exists so that the reference's own
// headers (nbdf_calculator.hpp, bdf_calculator.hpp, driftkick.hpp,
// chemmanager.hpp, saruprng.hpp, parameter.hpp) compile unmodified into the
// oracle/_ref harness. It is written from FDPS's public interface as the
// reference calls it (src/main.cpp:93-132, include/chemmanager.hpp:19-213,
// include/driftkick.hpp:43-54), not from FDPS source (FDPS is an un-vendored
// submodule, .gitmodules:1-3). Single process, single thread: the Comm
// collectives are the identity.
#pragma once

#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <random>
#include <vector>

namespace PS {

typedef int32_t S32;
typedef uint32_t U32;
typedef int64_t S64;
typedef uint64_t U64;
typedef float F32;
typedef double F64;

// Three-vector with the operator set the reference uses. Default construction
// zero-fills (the reference relies on it, e.g. bdf_calculator.hpp:156 Fbb[]).
template <class T>
struct Vector3 {
  T x, y, z;
  Vector3() : x(T(0)), y(T(0)), z(T(0)) {}
  Vector3(const T s) : x(s), y(s), z(s) {}
  Vector3(const T a, const T b, const T c) : x(a), y(b), z(c) {}

  Vector3& operator=(const T s) { x = y = z = s; return *this; }
  T& operator[](const int i) { return (&x)[i]; }
  const T& operator[](const int i) const { return (&x)[i]; }

  Vector3 operator+(const Vector3& v) const { return Vector3(x + v.x, y + v.y, z + v.z); }
  Vector3 operator-(const Vector3& v) const { return Vector3(x - v.x, y - v.y, z - v.z); }
  Vector3 operator-() const { return Vector3(-x, -y, -z); }
  // dot product, summed left to right
  T operator*(const Vector3& v) const { return x * v.x + y * v.y + z * v.z; }
  Vector3 operator*(const T s) const { return Vector3(x * s, y * s, z * s); }
  Vector3 operator/(const T s) const { return Vector3(x / s, y / s, z / s); }
  // cross product
  Vector3 operator^(const Vector3& v) const {
    return Vector3(y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x);
  }
  Vector3& operator+=(const Vector3& v) { x += v.x; y += v.y; z += v.z; return *this; }
  Vector3& operator-=(const Vector3& v) { x -= v.x; y -= v.y; z -= v.z; return *this; }
  Vector3& operator*=(const T s) { x *= s; y *= s; z *= s; return *this; }
  Vector3& operator/=(const T s) { x /= s; y /= s; z /= s; return *this; }
};
template <class T>
inline Vector3<T> operator*(const T s, const Vector3<T>& v) { return Vector3<T>(s * v.x, s * v.y, s * v.z); }

typedef Vector3<F64> F64vec;
typedef Vector3<F32> F32vec;

template <class T>
class ReallocatableArray {
  std::vector<T> d_;
 public:
  ReallocatableArray() {}
  explicit ReallocatableArray(const S32 n) { d_.reserve(n); }
  S32 size() const { return (S32)d_.size(); }
  S32 capacity() const { return (S32)d_.capacity(); }
  void resizeNoInitialize(const S32 n) { d_.resize(n); }
  void reserve(const S32 n) { d_.reserve(n); }
  void clearSize() { d_.clear(); }
  void push_back(const T& v) { d_.push_back(v); }
  void pushBackNoCheck(const T& v) { d_.push_back(v); }
  T& operator[](const S32 i) { return d_[i]; }
  const T& operator[](const S32 i) const { return d_[i]; }
  T* getPointer(const S32 i = 0) { return d_.data() + i; }
  const T* getPointer(const S32 i = 0) const { return d_.data() + i; }
};

template <class FP>
class ParticleSystem {
  std::vector<FP> p_;
 public:
  void initialize() {}
  void setNumberOfParticleLocal(const S32 n) { p_.resize(n); }
  S32 getNumberOfParticleLocal() const { return (S32)p_.size(); }
  S64 getNumberOfParticleGlobal() const { return (S64)p_.size(); }
  void ExpandParticleBuffer(const S32 n) { p_.reserve(n); }
  void AddNewParticle(const FP& fp) { p_.push_back(fp); }
  FP& operator[](const S32 i) { return p_[i]; }
  const FP& operator[](const S32 i) const { return p_[i]; }
  FP* getParticlePointer(const S32 i = 0) { return p_.data() + i; }
};

inline void Abort(const S32 = -1) { std::cerr << "PS::Abort\n"; std::abort(); }

struct Comm {
  static S32 getRank() { return 0; }
  static S32 getNumberOfProc() { return 1; }
  static S32 getThreadNum() { return 0; }
  static S32 getNumberOfThread() { return 1; }
  template <class T> static T getSum(const T& v) { return v; }
  template <class T> static T getMaxValue(const T& v) { return v; }
  template <class T> static void broadcast(T*, const S32, const S32 = 0) {}
  template <class T> static void exScan(const T*, T* out, const S32 n) {
    for (S32 i = 0; i < n; i++) out[i] = T(0);
  }
  template <class T> static void allGather(const T* in, const S32 n, T* out) {
    for (S32 i = 0; i < n; i++) out[i] = in[i];
  }
  template <class T> static void allGatherV(const T* in, const S32 n, T* out, const S32*, const S32*) {
    for (S32 i = 0; i < n; i++) out[i] = in[i];
  }
};

// FDPS's PS::MT is the Matsumoto-Nishimura mt19937ar generator; std::mt19937 is
// the same recurrence and seeding. real1 and real3 follow mt19937ar's
// genrand_real1 ([0,1]) and genrand_real3 ((0,1)).
struct MT {
  static std::mt19937& gen() { static std::mt19937 g(5489u); return g; }
  static void init_genrand(const unsigned long s) { gen().seed((uint32_t)s); }
  static uint32_t genrand_int32() { return (uint32_t)gen()(); }
  static double genrand_real1() { return genrand_int32() * (1.0 / 4294967295.0); }
  static double genrand_real3() { return (((double)genrand_int32()) + 0.5) * (1.0 / 4294967296.0); }
};

}  // namespace PS
