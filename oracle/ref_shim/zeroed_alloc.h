/*
 * Force-included (gcc -include) into the reference's sppde/sppde_core.c only.
 * The reference allocates every field with an uninitialised malloc
 * (sppde/sppde_core.c:193-203) and later reads a few cells it never writes
 * (the unset windy field, init.c:234; the psi/xi halo cells read by
 * laplacian_eta, laplacian.c:117-126). Zeroing allocations makes those reads
 * deterministic (0) without changing any value the reference writes.
 */
#include <stdlib.h>
#define malloc(n) calloc(1, (n))
