/* Exposes the reference's inline host helpers to Python (ctypes).
   TEST INFRASTRUCTURE: compiled together with the reference's own
   src/polygonal_light.c into oracle/_ref/libref_host.so. */
#include <stdint.h>
#include "math_utilities.h"

/* wang_random_number, math_utilities.h:50-57 */
uint32_t ref_wang_random_number(uint32_t seed) { return wang_random_number(seed); }
