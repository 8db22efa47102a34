// Link stub for oracle/_ref/libsfem_ref_f32.so: the reference's error path
// (SFEM_ERROR -> sfem_abort) resolved to abort().  Test infrastructure only.
#include <stdlib.h>

extern "C" void sfem_abort() { abort(); }
