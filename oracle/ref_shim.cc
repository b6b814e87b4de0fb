// ORACLE — test infrastructure only (never linked into the product).
//
// extern "C" shim around the reference's own host-compilable helpers. The reference
// writes its helpers so they compile as host C++ under -DGTEST (macro block at the top
// of each file, e.g. gaussian_helpers.cu:1-14); this file is compiled with the
// reference's helper directory on the include path, so the functions called below
// are the reference's code, unmodified:
//   math_helpers.cu:20-33    binomial_coefficient
//   math_helpers.cu:54-105   poz
//   math_helpers.cu:128-175  pchisq
//   set_helpers.cu:25-49     calculate_sepset_indices<level>
//   gaussian_helpers.cu      compute_m_2_inv<level> (cuPC Alg. 7), cholesky_decomposition,
//                            compute_inverse_matrix, gaussian_ci_test<level, n>
// The output goes to oracle/_ref/ only and is used to pin the C/numpy restatement.
#include "math_helpers.cu"
#include "set_helpers.cu"
#include "gaussian_helpers.cu"

// gaussian_ci_test<level, n> takes the variable count n as a template constant;
// the pin cases use correlation matrices of this fixed size.
static const int kRefPinP = 12;

extern "C" {

int ref_binomial(int n, int k) { return binomial_coefficient(n, k); }

double ref_poz(double z) { return poz(z); }

double ref_pchisq(double x, int df) { return pchisq(x, df); }

// level in 1..4; out receives `level` 1-based positions
int ref_sepset_indices(int level, int neighbours_count, int sepset_index, int *out) {
    switch (level) {
    case 1: calculate_sepset_indices<1>(neighbours_count, sepset_index, out); return 0;
    case 2: calculate_sepset_indices<2>(neighbours_count, sepset_index, out); return 0;
    case 3: calculate_sepset_indices<3>(neighbours_count, sepset_index, out); return 0;
    case 4: calculate_sepset_indices<4>(neighbours_count, sepset_index, out); return 0;
    default: return -1;
    }
}

// M (level x level, row-major) is copied first: compute_m_2_inv reads it only,
// but the copy keeps the caller's buffer untouched in every case.
int ref_m2_inv(int level, const double *M, double *out) {
    double tmp[64];
    for (int i = 0; i < level * level; ++i) tmp[i] = M[i];
    switch (level) {
    case 1: compute_m_2_inv<1>(tmp, out); return 0;
    case 2: compute_m_2_inv<2>(tmp, out); return 0;
    case 3: compute_m_2_inv<3>(tmp, out); return 0;
    case 4: compute_m_2_inv<4>(tmp, out); return 0;
    case 5: compute_m_2_inv<5>(tmp, out); return 0;
    case 6: compute_m_2_inv<6>(tmp, out); return 0;
    default: return -1;
    }
}

int ref_cholesky3(const double *A, double *L) {
    double tmp[9];
    for (int i = 0; i < 9; ++i) tmp[i] = A[i];
    cholesky_decomposition<3>(tmp, L);
    return 0;
}

int ref_inverse3(const double *A, double *out) {
    double tmp[9];
    for (int i = 0; i < 9; ++i) tmp[i] = A[i];
    compute_inverse_matrix<3>(tmp, out);
    return 0;
}

int ref_pin_p(void) { return kRefPinP; }

// One Gaussian CI test on a kRefPinP x kRefPinP correlation matrix C.
double ref_gaussian_ci_test(int level, unsigned vi, unsigned vj, double *C, int *sepset) {
    switch (level) {
    case 1: return gaussian_ci_test<1, kRefPinP>(vi, vj, C, sepset);
    case 2: return gaussian_ci_test<2, kRefPinP>(vi, vj, C, sepset);
    case 3: return gaussian_ci_test<3, kRefPinP>(vi, vj, C, sepset);
    case 4: return gaussian_ci_test<4, kRefPinP>(vi, vj, C, sepset);
    case 5: return gaussian_ci_test<5, kRefPinP>(vi, vj, C, sepset);
    case 6: return gaussian_ci_test<6, kRefPinP>(vi, vj, C, sepset);
    default: return -1.0;
    }
}

} // extern "C"
