/*
 * First-fit allocator over one device allocation, used by the request
 * server (serve.c) to place each job's buffers.  Offsets are relative to the
 * allocation; every block is rounded up to DMG_ARENA_ALIGN bytes; freed
 * blocks go back to an offset-sorted free list and merge with their
 * neighbours.  Not thread-safe: the server calls it under its mutex.
 * Header-only so that the CPU tests can compile it alone.
 */
#ifndef DMG_ARENA_H
#define DMG_ARENA_H
#include <stdlib.h>
#include <string.h>

#ifndef DMG_OK
#define DMG_OK 0
#endif
#ifndef DMG_ERR_NOMEM
#define DMG_ERR_NOMEM 4
#endif

#define DMG_ARENA_ALIGN 256

typedef struct {
  long long off, size;
} blk;

typedef struct {
  long long size, used;
  blk *free;
  int nfree, cap;
} arena;

static long long round_up(long long x) { return (x + DMG_ARENA_ALIGN - 1) / DMG_ARENA_ALIGN * DMG_ARENA_ALIGN; }

/* Offset of a block of at least `bytes` (rounded up) at the lowest free
 * offset that fits, or -1 when none does. */
static long long arena_alloc(arena *a, long long bytes) {
  bytes = round_up(bytes > 0 ? bytes : 1);
  for (int i = 0; i < a->nfree; ++i) {
    if (a->free[i].size >= bytes) {
      long long off = a->free[i].off;
      a->free[i].off += bytes;
      a->free[i].size -= bytes;
      if (a->free[i].size == 0) {
        memmove(&a->free[i], &a->free[i + 1], (size_t)(a->nfree - i - 1) * sizeof(blk));
        a->nfree--;
      }
      a->used += bytes;
      return off;
    }
  }
  return -1;
}

/* Return a block (the offset and size it was allocated with). */
static int arena_free(arena *a, long long off, long long bytes) {
  bytes = round_up(bytes > 0 ? bytes : 1);
  int i = 0;
  while (i < a->nfree && a->free[i].off < off) ++i;
  if (a->nfree == a->cap) {
    int nc = a->cap ? 2 * a->cap : 16;
    blk *nb = (blk *)realloc(a->free, (size_t)nc * sizeof(blk));
    if (!nb) return DMG_ERR_NOMEM;
    a->free = nb;
    a->cap = nc;
  }
  memmove(&a->free[i + 1], &a->free[i], (size_t)(a->nfree - i) * sizeof(blk));
  a->free[i].off = off;
  a->free[i].size = bytes;
  a->nfree++;
  /* coalesce with the neighbours */
  if (i + 1 < a->nfree && a->free[i].off + a->free[i].size == a->free[i + 1].off) {
    a->free[i].size += a->free[i + 1].size;
    memmove(&a->free[i + 1], &a->free[i + 2], (size_t)(a->nfree - i - 2) * sizeof(blk));
    a->nfree--;
  }
  if (i > 0 && a->free[i - 1].off + a->free[i - 1].size == a->free[i].off) {
    a->free[i - 1].size += a->free[i].size;
    memmove(&a->free[i], &a->free[i + 1], (size_t)(a->nfree - i - 1) * sizeof(blk));
    a->nfree--;
  }
  a->used -= bytes;
  return DMG_OK;
}

/* An arena of `size` bytes (rounded down to the alignment), empty; returns 0 or DMG_ERR_NOMEM. */
static int arena_init(arena *a, long long size) {
  memset(a, 0, sizeof(*a));
  a->size = size / DMG_ARENA_ALIGN * DMG_ARENA_ALIGN;
  a->cap = 16;
  a->free = (blk *)calloc(16, sizeof(blk));
  if (!a->free) return DMG_ERR_NOMEM;
  a->free[0].off = 0;
  a->free[0].size = a->size;
  a->nfree = a->size > 0;
  return DMG_OK;
}

static void arena_release(arena *a) {
  free(a->free);
  memset(a, 0, sizeof(*a));
}
#endif
