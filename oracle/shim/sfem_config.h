/* Type shim for compiling the reference CPU kernels standalone (oracle/_ref).
 * The numeric types follow the reference's default number selection
 * (cmake/SFEMNumbers.cmake:5-14): real/scalar/accumulator = double,
 * geom/jacobian = float32, idx/count/element_idx = int32, local_idx = int16.
 * Test infrastructure only. */
#ifndef SFEM_CONFIG_H
#define SFEM_CONFIG_H
#include <stdint.h>
#include <stddef.h>
#include <assert.h>
typedef double real_t;
typedef double scalar_t;
typedef double accumulator_t;
typedef float geom_t;
typedef float jacobian_t;
typedef float cu_jacobian_t;
typedef int32_t idx_t;
typedef int32_t count_t;
typedef int32_t element_idx_t;
typedef int16_t local_idx_t;
typedef uint32_t mask_t;
typedef uint16_t sshex8_count_t;
#define SFEM_IDX_INVALID (-1)
#define SFEM_LOG_LEVEL 0
#endif
