/* Run-length index sets (behaviour of reference index.c:7-60). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "index.h"

Index makeIndex(void) {
  Index ix = (Index)calloc(1, sizeof(struct index));
  if (!ix) return NULL;
  ix->size = INDEX_INITIAL_SIZE;
  ix->count = 0;
  ix->offsets = (int *)calloc(ix->size, sizeof(int));
  ix->counts = (int *)calloc(ix->size, sizeof(int));
  return ix;
}

void freeIndex(Index ix) {
  if (!ix) return;
  free(ix->offsets);
  free(ix->counts);
  free(ix);
}

/* Offsets arrive in increasing global-coordinate order; one that continues
 * the last run lengthens it, any other starts a new run. */
void addIndex(Index ix, int offset) {
  if (ix->count > 0) {
    int last = ix->count - 1;
    if (ix->offsets[last] + ix->counts[last] == offset) {
      ix->counts[last]++;
      return;
    }
  }
  if (ix->count == ix->size) {
    int nsize = ix->size * 2;
    int *no = (int *)realloc(ix->offsets, (size_t)nsize * sizeof(int));
    if (no) ix->offsets = no;
    int *nc = no ? (int *)realloc(ix->counts, (size_t)nsize * sizeof(int)) : NULL;
    if (nc) ix->counts = nc;
    if (!no || !nc) {
      dmg_error(DMG_ERR_NOMEM, "addIndex: out of host memory (%d runs)", ix->count);
      return; /* the index keeps its runs; the offset is not added */
    }
    ix->size = nsize;
  }
  ix->offsets[ix->count] = offset;
  ix->counts[ix->count] = 1;
  ix->count++;
}

void freeIndexList(Index *list) {
  if (!list) return;
  for (Index *p = list; *p != NULL; ++p) freeIndex(*p);
  free(list);
}

void printIndex(FILE *out, Index ix) {
  for (int r = 0; r < ix->count; ++r)
    for (int k = 0; k < ix->counts[r]; ++k) fprintf(out, "%d ", ix->offsets[r] + k);
}

void logIndex(Index ix) {
#ifdef DEBUG
  printIndex(stdout, ix);
#else
  (void)ix;
#endif
}

int sizeIndex(Index ix) {
  int n = 0;
  for (int r = 0; r < ix->count; ++r) n += ix->counts[r];
  return n;
}
