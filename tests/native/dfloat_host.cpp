// Host build of the double-float primitives used by the complex128 gate
// kernels (qcware_unitair_gb300/csrc/dfloat.cuh), exported for the CPU
// test that checks them against exact rational arithmetic.
#include "dfloat.cuh"

using namespace gbsv;

extern "C" {

void dfh_split(double x, float* out) {
  const DF d = df_split(x);
  out[0] = d.hi;
  out[1] = d.lo;
}

void dfh_entry(double x, float* out) {
  const DE d = df_entry(x);
  out[0] = d.hi;
  out[1] = d.mid;
  out[2] = d.lo;
}

double dfh_join(float hi, float lo) { return df_join(DF{hi, lo}); }

void dfh_fast2(float a, float b, float* out) {
  const DF d = df_fast2(a, b);
  out[0] = d.hi;
  out[1] = d.lo;
}

// y = M a for a 2x2 complex matrix (row-major, interleaved re/im) and an
// amplitude pair a = (a0, a1); form 0 = complex entries, 1 = real entries,
// 2 = RX form (real diagonal, imaginary off-diagonal), 3 = diagonal
// (complex), 4 = real diagonal, 5 = imaginary diagonal.
void dfh_gate(const double* m, const double* a, int form, double* y) {
  const DC a0 = df_split2(a[0], a[1]), a1 = df_split2(a[2], a[3]);
  DEC e[4];
  for (int j = 0; j < 4; ++j) e[j] = df_entry2(m[2 * j], m[2 * j + 1]);
  DC y0, y1;
  switch (form) {
    case 0:
      y0 = df_row2(e[0], a0, e[1], a1);
      y1 = df_row2(e[2], a0, e[3], a1);
      break;
    case 1:
      y0 = df_row2_real(e[0].re, a0, e[1].re, a1);
      y1 = df_row2_real(e[2].re, a0, e[3].re, a1);
      break;
    case 2:
      y0 = df_row2_rx(e[0].re, a0, e[1].im, a1);
      y1 = df_row2_rx(e[3].re, a1, e[2].im, a0);
      break;
    case 3:
      y0 = df_cmul(e[0], a0);
      y1 = df_cmul(e[3], a1);
      break;
    case 4:
      y0 = df_rmul(e[0].re, a0);
      y1 = df_rmul(e[3].re, a1);
      break;
    default:
      y0 = df_imul(e[0].im, a0);
      y1 = df_imul(e[3].im, a1);
      break;
  }
  y[0] = df_join(y0.re);
  y[1] = df_join(y0.im);
  y[2] = df_join(y1.re);
  y[3] = df_join(y1.im);
}

// y = M a for a 4x4 complex matrix (row-major, interleaved) and four
// amplitudes, row by row through df_row4.
void dfh_gate4(const double* m, const double* a, double* y) {
  DC av[4];
  for (int j = 0; j < 4; ++j) av[j] = df_split2(a[2 * j], a[2 * j + 1]);
  for (int row = 0; row < 4; ++row) {
    DEC e[4];
    for (int j = 0; j < 4; ++j)
      e[j] = df_entry2(m[8 * row + 2 * j], m[8 * row + 2 * j + 1]);
    const DC r = df_row4(e, av);
    y[2 * row] = df_join(r.re);
    y[2 * row + 1] = df_join(r.im);
  }
}

// y = M a for an 8x8 complex matrix (k = 3) through df_rowD<8>.
void dfh_gate8(const double* m, const double* a, double* y) {
  DC av[8];
  for (int j = 0; j < 8; ++j) av[j] = df_split2(a[2 * j], a[2 * j + 1]);
  for (int row = 0; row < 8; ++row) {
    DEC e[8];
    for (int j = 0; j < 8; ++j)
      e[j] = df_entry2(m[16 * row + 2 * j], m[16 * row + 2 * j + 1]);
    const DC r = df_rowD<8>(e, av);
    y[2 * row] = df_join(r.re);
    y[2 * row + 1] = df_join(r.im);
  }
}

void dfh_sincos(double theta, double* out) {
  const DSC r = df_sincos(theta);
  out[0] = df_join(r.s);
  out[1] = df_join(r.c);
}

}  // extern "C"
