/* Minimal stand-in for the reference's sfem_defs.hpp, which pulls in the
 * (absent) smesh submodule. Only what the compiled operator kernels use.
 * Test infrastructure only. */
#ifndef SFEM_DEFS_H
#define SFEM_DEFS_H
#include "sfem_base.hpp"
#include "sfem_macros.hpp"
#include <assert.h>
#include <string.h>
#endif
