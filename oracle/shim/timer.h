/* TEST INFRASTRUCTURE (oracle).  Declaration of the reference's timer.c
 * function (timer.c:8); the reference ships no timer.h. */
#ifndef ORACLE_SHIM_TIMER_H
#define ORACLE_SHIM_TIMER_H
double timer();
#endif
