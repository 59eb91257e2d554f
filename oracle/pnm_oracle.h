/* pnm oracle — C API of the CPU restatement in pnm_oracle.cpp.
 * TEST AND BASELINE INFRASTRUCTURE ONLY (never linked into the product library).
 * Dims are (nx, ny, nz) with x fastest; origin/spacing are xyz float32; grad_p is xyz float64. */
#ifndef PNM_ORACLE_H
#define PNM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  float x, y, z, radius;
} pnmo_pore;

typedef struct {
  int64_t n_pores, n_throats;
  pnmo_pore* pores;
  double* pore_pressure;
  double* pore_residual;
  int32_t* throats; /* 2 * n_throats */
  double* throat_flow;
  double* throat_area;
  double* throat_dp;
  long long* throat_root; /* patch root face id per throat */
  int32_t* pore_peak;     /* basin peak voxel per pore label (0 when none) */
  double* throat_absflow; /* sum of |q| over the faces of each throat (tolerance scale) */
  double* pore_absflux;   /* sum of |q| over the faces each pore residual sums */
} pnmo_flow_result;

void pnmo_free(void* p);
int64_t pnmo_extract_pores(const float* sdf, int nx, int ny, int nz, const float* origin,
                           const float* spacing, pnmo_pore** pores, int threads);
void pnmo_segment_volume(const float* sdf, int nx, int ny, int nz, const float* spacing,
                         int32_t* seg, int32_t* roots, int threads);
int64_t pnmo_extract_topology(const int32_t* seg, int nx, int ny, int nz, int32_t** pairs,
                              int threads);
void pnmo_extract_pore_network(const float* sdf, int nx, int ny, int nz, const float* origin,
                               const float* spacing, pnmo_pore** pores, int64_t* n_pores,
                               int32_t* seg, int32_t** pairs, int64_t* n_pairs, int threads);
pnmo_flow_result* pnmo_extract_network_flow(const float* sdf, int nx, int ny, int nz,
                                            const float* origin, const float* spacing,
                                            const double* u, const double* v, const double* w,
                                            const double* p, const double* ox, const double* oy,
                                            const double* oz, const double* grad_p, int threads);
void pnmo_flow_result_free(pnmo_flow_result* r);

#ifdef __cplusplus
}
#endif
#endif
