/*
 * hthread_host.h -- the MT-3000 host runtime interface the reference's host
 * programs use, implemented on the GB300 library, so those programs build
 * and run unmodified against libgbblas (link -lgbblas).
 *
 * Covers what the reference demos call (e.g.
 * sgemm_release_V1.3.2/host_code/sgemm_demo.c:50-61, :93-94, :128-145,
 * :338-351): device open/close, kernel-image load, device malloc/free,
 * barrier ids, thread groups and launch by name.  Mapping:
 *   hthread_malloc       -> CUDA managed memory (the demos fill and check
 *                           buffers on the host and hand them to the device)
 *   hthread_group_exec   -> gb_exec (kernel name + scalars-then-pointers)
 *   hthread_group_wait   -> gb_sync
 *   dat_load, barriers, group create/destroy -> bookkeeping only (the kernels
 *                           are linked into the library; a GPU needs no
 *                           thread-group or barrier setup).
 * The cluster id selects nothing: everything runs on the current CUDA device.
 */
#ifndef GB_HTHREAD_HOST_H
#define GB_HTHREAD_HOST_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HT_MEM_RO 0
#define HT_MEM_WO 1
#define HT_MEM_RW 2

int   hthread_dev_open(int dev_id);
void  hthread_dev_close(int dev_id);
int   hthread_dat_load(int dev_id, const char *image_name);
void *hthread_malloc(int dev_id, size_t bytes, int flag);
void  hthread_free(void *ptr);
int   hthread_barrier_create(int dev_id);
void  hthread_barrier_destroy(int barrier_id);
int   hthread_group_create(int dev_id, int nthreads);
int   hthread_group_exec(int group_id, const char *kernel_name, int n_scalar, int n_ptr, unsigned long *args);
int   hthread_group_wait(int group_id);
void  hthread_group_destroy(int group_id);

#ifdef __cplusplus
}
#endif
#endif
