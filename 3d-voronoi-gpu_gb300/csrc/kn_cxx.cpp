// C++-linkage exports of the kn_* API.
//
// The reference's knearests.h (knearests.h:20-27) declares kn_prepare,
// kn_solve, kn_free, kn_print_stats and kn_get_* without extern "C", so an
// object compiled against that header calls the C++-mangled names
// (_Z10kn_prepareP6float3i, ...).  include/knearests.h declares the same
// functions with C linkage.  This file exports both: each C++-linkage
// function below forwards to its C-linkage twin (kn_api.cu), so objects built
// against either header link against this library unchanged.
//
// The C functions are reached through declarations whose assembler names are
// the C symbols; the header is included with its function names renamed so
// that only its kn_problem type is used here (its mangled name, 10kn_problem,
// is the reference's: a typedef of an unnamed struct).
#define kn_prepare vgb_hdr_kn_prepare
#define kn_solve vgb_hdr_kn_solve
#define kn_free vgb_hdr_kn_free
#define kn_print_stats vgb_hdr_kn_print_stats
#define kn_get_points vgb_hdr_kn_get_points
#define kn_get_knearests vgb_hdr_kn_get_knearests
#define kn_get_permutation vgb_hdr_kn_get_permutation
#include "../../include/knearests.h"
#undef kn_prepare
#undef kn_solve
#undef kn_free
#undef kn_print_stats
#undef kn_get_points
#undef kn_get_knearests
#undef kn_get_permutation

namespace vgb_c_abi {
kn_problem* c_kn_prepare(float3* points, int numpoints) __asm__("kn_prepare");
void c_kn_solve(kn_problem* kn) __asm__("kn_solve");
void c_kn_free(kn_problem** kn) __asm__("kn_free");
void c_kn_print_stats(kn_problem* kn) __asm__("kn_print_stats");
float3* c_kn_get_points(kn_problem* kn) __asm__("kn_get_points");
unsigned int* c_kn_get_knearests(kn_problem* kn) __asm__("kn_get_knearests");
unsigned int* c_kn_get_permutation(kn_problem* kn) __asm__("kn_get_permutation");
}  // namespace vgb_c_abi
using namespace vgb_c_abi;

__attribute__((visibility("default"))) kn_problem* kn_prepare(float3* points, int numpoints) {
  return c_kn_prepare(points, numpoints);
}
__attribute__((visibility("default"))) void kn_solve(kn_problem* kn) { c_kn_solve(kn); }
__attribute__((visibility("default"))) void kn_free(kn_problem** kn) { c_kn_free(kn); }
__attribute__((visibility("default"))) void kn_print_stats(kn_problem* kn) { c_kn_print_stats(kn); }
__attribute__((visibility("default"))) float3* kn_get_points(kn_problem* kn) { return c_kn_get_points(kn); }
__attribute__((visibility("default"))) unsigned int* kn_get_knearests(kn_problem* kn) {
  return c_kn_get_knearests(kn);
}
__attribute__((visibility("default"))) unsigned int* kn_get_permutation(kn_problem* kn) {
  return c_kn_get_permutation(kn);
}
