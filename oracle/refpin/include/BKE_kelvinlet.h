/* Stand-in for a header the reference does not ship (kelvinlet.c includes it):
 * the Kelvinlet parameter block and entry points as kelvinlet.c uses them. */
#include "refpin_prelude.h"

#define KELVINLET_MAX_ITERATIONS 3

typedef struct KelvinletParams {
  float a;
  float b;
  float c;
  float f;
  float radius_scaled[KELVINLET_MAX_ITERATIONS];
} KelvinletParams;

void BKE_kelvinlet_init_params(
    KelvinletParams *params, float radius, float force, float shear_modulus, float poisson_ratio);
void BKE_kelvinlet_grab(float radius_elem_disp[3], const KelvinletParams *params,
                        const float elem_orig_co[3], const float brush_location[3],
                        const float brush_delta[3]);
void BKE_kelvinlet_grab_biscale(float radius_elem_disp[3], const KelvinletParams *params,
                                const float elem_orig_co[3], const float brush_location[3],
                                const float brush_delta[3]);
void BKE_kelvinlet_grab_triscale(float radius_elem_disp[3], const KelvinletParams *params,
                                 const float elem_orig_co[3], const float brush_location[3],
                                 const float brush_delta[3]);
void BKE_kelvinlet_scale(float radius_elem_disp[3], const KelvinletParams *params,
                         const float elem_orig_co[3], const float brush_location[3],
                         const float surface_normal[3]);
void BKE_kelvinlet_twist(float radius_elem_disp[3], const KelvinletParams *params,
                         const float elem_orig_co[3], const float brush_location[3],
                         const float surface_normal[3]);
