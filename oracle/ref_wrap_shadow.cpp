// Compiles the reference's shadow lookups (src/shaders/shadow.cpp) unmodified,
// from where it lies, with three build-time selections made by this wrapper:
//   FR_SHADOW_MODE 0 = hard shadow, 1 = PCF, 2 = PCSS (the reference's default);
//   the PCF / blocker-search tap counts come from runtime globals of the harness;
//   with FR_TABLE_RNG the disk draws read the deterministic tables of
//   include/fr_sample_tables.h instead of the global mt19937 stream.
// shadow.h uses #pragma once, so re-including it from shadow.cpp is a no-op and
// the overrides below stay in force for the body of shadow.cpp.
#include "shadow.h"

extern int fr_ref_pcf_samples;
extern int fr_ref_blocker_samples;

#undef PCF_NUM_SAMPLES
#undef PCSS_BLOCKER_SEARCH_NUM_SAMPLES
#define PCF_NUM_SAMPLES fr_ref_pcf_samples
#define PCSS_BLOCKER_SEARCH_NUM_SAMPLES fr_ref_blocker_samples

#ifndef FR_SHADOW_MODE
#define FR_SHADOW_MODE 2
#endif
#if FR_SHADOW_MODE == 0
#undef SOFT_SHADOW_PCSS
#undef SOFT_SHADOW_PCF
#elif FR_SHADOW_MODE == 1
#undef SOFT_SHADOW_PCSS
#define SOFT_SHADOW_PCF
#endif

#ifdef FR_TABLE_RNG
Vector3f fr_ref_disk_sample(const char* caller);
#define RandomVectorInUnitDisk() fr_ref_disk_sample(__func__)
#endif

#include "shaders/shadow.cpp"
