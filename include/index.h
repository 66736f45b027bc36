#ifndef INDEX_H
#define INDEX_H
/**
 * @file index.h
 * Run-length index sets: the local offsets of one axis, kept as
 * (offset, count) runs.  Same struct and functions as the reference's
 * index.h:8-24; adjacent offsets appended in order merge into one run
 * (reference index.c:23-42).
 */
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

struct index {
  int size;     /**< capacity of offsets/counts */
  int count;    /**< number of runs */
  int *offsets; /**< first offset of each run */
  int *counts;  /**< length of each run */
};
typedef struct index *Index;

#define INDEX_INITIAL_SIZE 16

/** Empty index (reference index.h:19). */
Index makeIndex(void);
/** Free an index (reference index.h:20). */
void freeIndex(Index);
/** Append one offset, extending the last run when it is contiguous
 * (reference index.h:21). */
void addIndex(Index i, int offset);
/** Free a NULL-terminated array of indexes (reference index.h:22). */
void freeIndexList(Index *list);
/** Print every offset (reference index.h:23). */
void printIndex(FILE *out, Index index);
/** Debug-log every offset (reference index.h:24); silent unless built with -DDEBUG. */
void logIndex(Index index);
/** Total number of offsets in the index (sum of the run counts). */
int sizeIndex(Index index);

#ifdef __cplusplus
}
#endif
#endif
