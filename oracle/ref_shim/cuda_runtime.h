/* Empty stand-in: fluid_system_cuda.cuh includes cuda_runtime.h; the pinned kernels need nothing from it. */
