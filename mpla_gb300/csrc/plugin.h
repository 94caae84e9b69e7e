// Plugin-side helpers: turning a kernel_matrix_data descriptor or a
// system_assembler object into a GaussSystem for the fused kernels.
#pragma once

#include "../../include/mpla.h"
#include "../../include/kernel.h"
#include "internal.h"

namespace mgb {

// kernel.h descriptor (host struct, device array of device pointers).
int kernel_data_system(const kernel_matrix_data* kd, const mpla_generic_matrix* A, GaussSystem* g);
// Device object created by this library's Gaussian assembler factory;
// returns MGB_ERR_ARG for any other object.
int assembler_system(const void* dev_object, const mpla_generic_matrix* A, GaussSystem* g);
// Fused matvec that evaluates an arbitrary system_assembler through its
// virtual get_matrix_entry (object constructed in this library's module).
Matvec* new_generic_assembler_matvec(DeviceContext* c, mpla_generic_matrix* A);

}  // namespace mgb
