// Test stand-in for the parts of eQ's src/eQ.h that the drop-in fHSL.h binds to, for
// machines without the reference sources (its JSON library included): the plugin
// base class eQ::diffusionSolver with its params (src/eQ.h:302-330), eQ::gridFunction
// (src/eQ.h:34-86), eQ::data::ij_from_xy (src/eQ.h:119-130) and the parameter store,
// here a minimal JSON value with the operations the drop-in and the test driver use.
// Test infrastructure only.
#pragma once
#include <cmath>
#include <cstddef>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#define EQ_TEST_STANDIN 1
typedef int MPI_Comm;

namespace eqmock {

class Json {
 public:
  enum Kind { NUL, NUM, STR, ARR, OBJ };
  Json() = default;
  Json(double v) : kind_(NUM), num_(v) {}
  Json(int v) : kind_(NUM), num_(v) {}
  Json(const char* s) : kind_(STR), str_(s) {}
  Json(const std::string& s) : kind_(STR), str_(s) {}
  Json(const std::vector<double>& v) : kind_(ARR) {
    for (double x : v) arr_.push_back(Json(x));
  }
  static Json array(std::vector<Json> items) {
    Json j;
    j.kind_ = ARR;
    j.arr_ = std::move(items);
    return j;
  }
  Json& operator[](const std::string& k) {
    if (kind_ == NUL) kind_ = OBJ;
    if (kind_ != OBJ) throw std::runtime_error("not an object");
    for (auto& e : obj_)
      if (e.first == k) return e.second;
    obj_.emplace_back(k, Json());
    return obj_.back().second;
  }
  Json& operator[](const char* k) { return (*this)[std::string(k)]; }
  Json& operator[](int i) { return arr_.at((size_t)i); }
  std::size_t count(const std::string& k) const {
    if (kind_ != OBJ) return 0;
    for (const auto& e : obj_)
      if (e.first == k) return 1;
    return 0;
  }
  template <class T>
  T get() const;

 private:
  Kind kind_ = NUL;
  double num_ = 0.0;
  std::string str_;
  std::vector<Json> arr_;
  std::vector<std::pair<std::string, Json>> obj_;
};

template <>
inline double Json::get<double>() const {
  if (kind_ != NUM) throw std::runtime_error("not a number");
  return num_;
}
template <>
inline std::string Json::get<std::string>() const {
  if (kind_ != STR) throw std::runtime_error("not a string");
  return str_;
}
template <>
inline std::vector<double> Json::get<std::vector<double>>() const {
  if (kind_ != ARR) throw std::runtime_error("not an array");
  std::vector<double> v;
  for (const auto& e : arr_) v.push_back(e.get<double>());
  return v;
}

}  // namespace eqmock

namespace eQ {

using nodePoint = std::pair<size_t, size_t>;

template <class T>
class gridFunction {
 public:
  gridFunction(size_t nh, size_t nw) : nw_(nw), g_(nh * nw, T(0)) {}
  T& operator[](const nodePoint& p) { return g_[p.first * nw_ + p.second]; }

 private:
  size_t nw_;
  std::vector<T> g_;
};

class data {
 public:
  using parametersType = eqmock::Json;
  using files_t = std::vector<int>;
  static parametersType parameters;
  static inline std::pair<size_t, size_t> ij_from_xy(double x, double y, double n) {
    return std::make_pair(size_t(std::round(y * n)), size_t(std::round(x * n)));
  }
};

class diffusionSolver {
 public:
  struct params {
    int argc;
    char** argv;
    size_t uniqueID;
    MPI_Comm comm;
    double dt;
    double D_HSL;
    std::string filePath;
    std::string filePathTopChannel;
    std::string filePathBottomChannel;
    std::shared_ptr<eQ::data::files_t> dataFiles;
    double trapHeightMicrons;
    double trapWidthMicrons;
    double nodesPerMicron;
    double trapChannelVelocity;
  };
  virtual void initDiffusion(eQ::diffusionSolver::params&) = 0;
  virtual void stepDiffusion() {}
  virtual eQ::data::parametersType getBoundaryFlux(void) { return {}; }
  virtual void writeDiffusionFiles(double timestamp) = 0;
  virtual void finalize(void) {}
  virtual ~diffusionSolver() = default;
};

}  // namespace eQ
