/*
 * hthread_shim.c -- the reference host runtime interface (hthread_host.h)
 * on top of the GB300 library: reference host programs run unmodified.
 * Return conventions follow the demos' use: 0 on success, -1 on failure;
 * the library status of the failing call stays in gb_get_last_status().
 */
#include "hthread_host.h"

#include "gbblas.h"

static int g_barriers = 0;

int hthread_dev_open(int dev_id) { (void)dev_id; return gb_device_arch() > 0 ? 0 : -1; }
void hthread_dev_close(int dev_id) { (void)dev_id; gb_sync(0); }
int hthread_dat_load(int dev_id, const char *image_name) { (void)dev_id; (void)image_name; return 0; }

void *hthread_malloc(int dev_id, size_t bytes, int flag)
{
    void *p = 0;
    (void)dev_id; (void)flag;
    return gb_malloc_managed(&p, bytes) == GB_OK ? p : 0;
}

void hthread_free(void *ptr) { gb_free(ptr); }
int hthread_barrier_create(int dev_id) { (void)dev_id; return g_barriers++; }
void hthread_barrier_destroy(int barrier_id) { (void)barrier_id; }
int hthread_group_create(int dev_id, int nthreads) { (void)dev_id; (void)nthreads; return 1; }
void hthread_group_destroy(int group_id) { (void)group_id; }

int hthread_group_exec(int group_id, const char *kernel_name, int n_scalar, int n_ptr, unsigned long *args)
{
    (void)group_id;
    return gb_exec(kernel_name, n_scalar, n_ptr, args) == GB_OK ? 0 : -1;
}

int hthread_group_wait(int group_id) { (void)group_id; return gb_sync(0) == GB_OK ? 0 : -1; }
