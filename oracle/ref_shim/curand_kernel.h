/* Empty stand-in: fluid_system_cuda.cuh includes curand_kernel.h; the pinned kernels need nothing from it. */
