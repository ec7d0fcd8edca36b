// A number type over double-float arithmetic (dfloat.cuh), so that templated straight-line
// code (mf_contract.cuh) can be evaluated with ~48-bit accuracy on the FP32 pipe.
#pragma once
#include "dfloat.cuh"

namespace ibem {

struct DF {
  dfloat v;
  IBEM_HD DF() : v{0.0f, 0.0f} {}
  IBEM_HD DF(double x) : v(df_make(x)) {}
  IBEM_HD explicit DF(dfloat d) : v(d) {}
};

IBEM_HD inline DF operator+(DF a, DF b) { return DF(a.v + b.v); }
IBEM_HD inline DF operator-(DF a, DF b) { return DF(a.v - b.v); }
IBEM_HD inline DF operator-(DF a) { return DF(-a.v); }
IBEM_HD inline DF operator*(DF a, DF b) { return DF(a.v * b.v); }
IBEM_HD inline DF& operator+=(DF& a, DF b) {
  a.v = a.v + b.v;
  return a;
}
IBEM_HD inline bool operator>(DF a, DF b) { return a.v.hi > b.v.hi || (a.v.hi == b.v.hi && a.v.lo > b.v.lo); }

// x^-1/2: FP32 estimate and one double-float Newton step
IBEM_HD inline DF rsqrt_t(DF x) {
  float y0;
#ifdef __CUDA_ARCH__
  y0 = rsqrtf(x.v.hi);
#else
  y0 = 1.0f / std::sqrt(x.v.hi);
#endif
  const dfloat yd{y0, 0.0f};
  const dfloat t = dfloat{1.0f, 0.0f} - x.v * (yd * yd);
  return DF(yd + yd * (t * 0.5f));
}

IBEM_HD inline double df_value(DF a) { return (double)a.v.hi + (double)a.v.lo; }

}  // namespace ibem
