/* Drives the request server's arena (arena.h) from commands on stdin, for
 * tests/test_arena.py:
 *   i <size>          make the arena
 *   a <bytes>         allocate: prints the offset (-1 when nothing fits)
 *   f <off> <bytes>   free: prints the status
 *   s                 prints "used <n> free <off>:<size> ..." */
#include <stdio.h>
#include "arena.h"

int main(void) {
  arena ar;
  int made = 0;
  char op;
  while (scanf(" %c", &op) == 1) {
    long long x = 0, y = 0;
    if (op == 'i' && scanf("%lld", &x) == 1) {
      if (made) arena_release(&ar);
      made = arena_init(&ar, x) == DMG_OK;
      printf("%lld\n", made ? ar.size : -1);
    } else if (op == 'a' && scanf("%lld", &x) == 1) {
      printf("%lld\n", arena_alloc(&ar, x));
    } else if (op == 'f' && scanf("%lld %lld", &x, &y) == 2) {
      printf("%d\n", arena_free(&ar, x, y));
    } else if (op == 's') {
      printf("used %lld free", ar.used);
      for (int i = 0; i < ar.nfree; ++i) printf(" %lld:%lld", ar.free[i].off, ar.free[i].size);
      printf("\n");
    } else {
      return 2;
    }
    fflush(stdout);
  }
  if (made) arena_release(&ar);
  return 0;
}
