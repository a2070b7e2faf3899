// Compiles the reference's frame orchestration (src/render.cpp) unmodified, from
// where it lies. With FR_TABLE_RNG the SSAO hemisphere draw of pixel (x, y),
// sample s (render.cpp:240) reads the deterministic tables of
// include/fr_sample_tables.h instead of the global mt19937 stream; x, y and s are
// the loop variables of Render::DoSSAO at that call site.
#include "render.h"

#ifdef FR_TABLE_RNG
Vector3f fr_ref_hemisphere_sample(const Vector3f& normal, int x, int y, int s);
#define RandomVectorInHemisphere(n) fr_ref_hemisphere_sample((n), x, y, s)
#endif

#include "render.cpp"
