/* Test-infrastructure stub (oracle build only): the MSVC aligned allocator the
 * reference's memory.hxx calls, mapped onto posix_memalign. Not product code. */
#pragma once
#include_next <malloc.h>
#include <stdlib.h>
static inline void *_aligned_malloc(size_t size, size_t alignment)
{
    void *p = NULL;
    if (alignment < sizeof(void *)) alignment = sizeof(void *);
    if (posix_memalign(&p, alignment, size ? size : alignment) != 0) return NULL;
    return p;
}
static inline void _aligned_free(void *p) { free(p); }
