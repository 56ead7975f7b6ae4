/*
 * hthread_host.h -- a stand-in for the MT-3000 host runtime header, used
 * ONLY to compile the reference's own host demo programs (their CPU check
 * loops are the ground truth the oracle is pinned against).  TEST
 * INFRASTRUCTURE: nothing in the product includes this file.
 *
 * The demos include <stdlib.h> before this header, so the three macros at
 * the end apply only to the demo's own code:
 *   malloc -> records host buffers (the CPU check's result array),
 *   rand/srand -> a reproducible counter-based stream, so the inputs the
 *                 demo generates can be regenerated bit-for-bit by the tests.
 * hthread_group_exec dispatches the device kernel name to the oracle
 * (oracle.c), so the demo's own element-wise check compares the oracle
 * with the reference loop.  hthread_dev_close dumps every buffer to the
 * file named by $GBREF_DUMP.
 */
#ifndef GBREF_HTHREAD_HOST_H
#define GBREF_HTHREAD_HOST_H

#include <stddef.h>

#define HT_MEM_RO 0
#define HT_MEM_WO 1
#define HT_MEM_RW 2

int   hthread_dev_open(int dev_id);
int   hthread_dat_load(int dev_id, const char *name);
void *hthread_malloc(int dev_id, size_t size, int flag);
void  hthread_free(void *ptr);
int   hthread_barrier_create(int dev_id);
void  hthread_barrier_destroy(int bid);
int   hthread_group_create(int dev_id, int nthreads);
int   hthread_group_wait(int tg_id);
int   hthread_group_exec(int tg_id, const char *name, int n_scalar, int n_ptr, unsigned long *args);
void  hthread_group_destroy(int tg_id);
void  hthread_dev_close(int dev_id);

void *gbref_host_malloc(size_t n);
int   gbref_rand(void);
void  gbref_srand(unsigned seed);

#define malloc(n) gbref_host_malloc(n)
#define rand() gbref_rand()
#define srand(s) gbref_srand(s)

#endif
