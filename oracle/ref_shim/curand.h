/* Empty stand-in: fluid_system_cuda.cuh includes curand.h; the pinned kernels need nothing from it. */
