// Host build of the double-float routines used by the far-field tiles
// (bem_gmsh_gb300/csrc/df32.cuh).  Compiled by tests/test_df32_cpu.py with
// floating-point contraction off, so every result is bit-identical to the
// device code; the test compares them with long-double references.
#include "../../bem_gmsh_gb300/csrc/df32.cuh"

extern "C" {

void df_log_batch(const double* x, int n, double* out) {
  df::LogEntry tab[df::kLogTable];
  for (int i = 0; i < df::kLogTable; ++i) tab[i] = df::log_entry(i);
  for (int i = 0; i < n; ++i) out[i] = df::to_double(df::log(df::from_double(x[i]), tab));
}

void df_div_batch(const double* a, const double* b, int n, double* out) {
  for (int i = 0; i < n; ++i) out[i] = df::to_double(df::div(df::from_double(a[i]), df::from_double(b[i])));
}

void df_mul_batch(const double* a, const double* b, int n, double* out) {
  for (int i = 0; i < n; ++i) out[i] = df::to_double(df::mul(df::from_double(a[i]), df::from_double(b[i])));
}

void df_to_double_batch(const float* h, const float* l, int n, double* out) {
  for (int i = 0; i < n; ++i) out[i] = df::to_double(df::f2{h[i], l[i]});
}

// xn - xs through the three-float splits
void df_diff_batch(const double* xn, const double* xs, int n, double* out) {
  for (int i = 0; i < n; ++i) {
    float an, bn, cn, as, bs, cs;
    df::split3(xn[i], an, bn, cn);
    df::split3(xs[i], as, bs, cs);
    out[i] = df::to_double(df::diff3(an, bn, cn, as, bs, cs));
  }
}

}

extern "C" {

// (float)(v * 2^s) on the integer path of the equilibration kernel
void df_scale_to_f32_batch(const double* v, const int* s, int n, float* out) {
  for (int i = 0; i < n; ++i) out[i] = df::scale_to_f32(v[i], s[i]);
}

}
