/* Stand-in for the reference's missing randCL_well512.cl (fluid.h includes it for the state
 * type of its OpenCL random generator, which the pinned kernels do not use). */
#ifndef MG_REF_SHIM_WELL512
#define MG_REF_SHIM_WELL512
typedef struct well512_state { unsigned int s[16]; unsigned int i; } well512_state;
#endif
