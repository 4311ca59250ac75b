// A minimal stand-in for the part of AMReX's interface that
// include/AmrDG_GB300.h uses (Box, BoxArray, FArrayBox, MultiFab, MFIter,
// Abort), with FArrayBox data in device memory as in an AMReX GPU build.
// Test infrastructure only.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#ifndef AMREX_SPACEDIM
#define AMREX_SPACEDIM 2
#endif

namespace amrex {

[[noreturn]] inline void Abort(const std::string& msg) { throw std::runtime_error(msg); }

struct Box {
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  int smallEnd(int d) const { return lo[d]; }
  int bigEnd(int d) const { return hi[d]; }
  int length(int d) const { return hi[d] - lo[d] + 1; }
  long long numPts() const {
    long long n = 1;
    for (int d = 0; d < AMREX_SPACEDIM; ++d) n *= length(d);
    return n;
  }
  Box grown(int g) const {
    Box b = *this;
    for (int d = 0; d < AMREX_SPACEDIM; ++d) {
      b.lo[d] -= g;
      b.hi[d] += g;
    }
    return b;
  }
};

struct BoxArray {
  std::vector<Box> boxes;
  int size() const { return (int)boxes.size(); }
  Box operator[](int i) const { return boxes[i]; }
};

// Fortran-ordered data over the grown box, components slowest.
struct FArrayBox {
  Box bx;
  int ncomp = 0;
  double* d = nullptr;
  const Box& box() const { return bx; }
  double* dataPtr() { return d; }
  int nComp() const { return ncomp; }
};

class MultiFab;

class MFIter {
 public:
  explicit MFIter(const MultiFab& mf) : mf_(&mf) {}
  bool isValid() const;
  MFIter& operator++() {
    ++i_;
    return *this;
  }
  Box validbox() const;
  int index() const { return i_; }

 private:
  const MultiFab* mf_;
  int i_ = 0;
};

class MultiFab {
 public:
  MultiFab() = default;
  MultiFab(const MultiFab&) = delete;
  MultiFab& operator=(const MultiFab&) = delete;
  ~MultiFab() {
    for (auto& f : fabs_)
      if (f.d) cudaFree(f.d);
  }
  void define(const BoxArray& ba, int ncomp, int ngrow) {
    ba_ = ba;
    ng_ = ngrow;
    for (const Box& b : ba.boxes) {
      FArrayBox f;
      f.bx = b.grown(ngrow);
      f.ncomp = ncomp;
      if (cudaMalloc(&f.d, (size_t)f.bx.numPts() * ncomp * sizeof(double)) != cudaSuccess) Abort("cudaMalloc");
      fabs_.push_back(f);
    }
  }
  int nGrow() const { return ng_; }
  const BoxArray& boxArray() const { return ba_; }
  FArrayBox& operator[](const MFIter& mfi) { return fabs_[mfi.index()]; }
  FArrayBox& fab(int i) { return fabs_[i]; }
  int nfabs() const { return (int)fabs_.size(); }

 private:
  BoxArray ba_;
  int ng_ = 0;
  std::vector<FArrayBox> fabs_;
};

inline bool MFIter::isValid() const { return i_ < mf_->boxArray().size(); }
inline Box MFIter::validbox() const { return mf_->boxArray()[i_]; }

}  // namespace amrex
