/* ORACLE -- test infrastructure.  A header-only stand-in for the few HDF5
 * calls the reference's generated solver makes, so that it compiles here
 * without libhdf5.  A "file" is a directory <path>.d holding one raw
 * little-endian float64 file <dataset>.f64 per dataset and @<name>.f64 per
 * attribute.  If the environment variable DGO_REF_TABLE_DIR is set,
 * relative paths are resolved in it. */
#ifndef DGO_HDF5_SHIM_H
#define DGO_HDF5_SHIM_H
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
#define H5F_ACC_RDONLY 0
#define H5F_ACC_TRUNC 1
#define H5P_DEFAULT 0

#define DGO_SHIM_MAXF 64
static char dgo_shim_paths[DGO_SHIM_MAXF][1024];
static int dgo_shim_next = 0;

static inline hid_t H5Fopen(const char *name, unsigned flags, hid_t plist)
{
    (void)flags; (void)plist;
    int id = dgo_shim_next++ % DGO_SHIM_MAXF;
    const char *dir = getenv("DGO_REF_TABLE_DIR");
    if (dir && name[0] != '/')
        snprintf(dgo_shim_paths[id], sizeof(dgo_shim_paths[id]), "%s/%s.d", dir, name);
    else
        snprintf(dgo_shim_paths[id], sizeof(dgo_shim_paths[id]), "%s.d", name);
    return id;
}
static inline hid_t H5Fcreate(const char *name, unsigned f, hid_t a, hid_t b)
{
    (void)a; (void)b;
    const hid_t id = H5Fopen(name, f, 0);
    mkdir(dgo_shim_paths[id], 0755);
    return id;
}
static inline herr_t H5Fclose(hid_t id) { (void)id; return 0; }
#endif
