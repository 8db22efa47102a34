/* Type shim for the reference's float32 number configuration (oracle/_ref).
 * Same as oracle/shim/sfem_config.h except real/scalar/accumulator = float,
 * the selection SFEM_REAL_TYPE=float32 makes (cmake/SFEMNumbers.cmake:5-10).
 * Test infrastructure only. */
#ifndef SFEM_CONFIG_H
#define SFEM_CONFIG_H
#include <stdint.h>
#include <stddef.h>
#include <assert.h>
typedef float real_t;
typedef float scalar_t;
typedef float accumulator_t;
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
