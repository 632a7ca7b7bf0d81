/*
 * Minimal stand-in for <hdf5.h>, used only to compile the reference's
 * hot-path sources into the oracle harness (oracle/ref/Makefile).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  The HDF5 library is not installed in
 * the build container; the hot path (actions + SPopulation step) never
 * touches a file, it only mentions HDF5 types and calls in its QDF
 * dump/restore methods, which the harness never invokes.  Every function
 * here is a no-op that reports failure, so an accidental call cannot
 * silently pretend to succeed.
 *
 * Written from scratch; it copies nothing from the HDF5 sources (only the
 * public identifier names the reference code spells out).
 */
#ifndef QHG_ORACLE_HDF5_SHIM_H
#define QHG_ORACLE_HDF5_SHIM_H

#include <stddef.h>
#include <stdint.h>

typedef int64_t            hid_t;
typedef unsigned long long hsize_t;
typedef long long          hssize_t;
typedef int                herr_t;
typedef int                htri_t;
typedef bool               hbool_t;

#define HOFFSET(S, M) (offsetof(S, M))

/* property / selection constants */
#define H5P_DEFAULT     ((hid_t)0)
#define H5S_ALL         ((hid_t)0)
#define H5S_SELECT_SET  0
#define H5F_ACC_RDONLY  0u
#define H5F_ACC_RDWR    1u
#define H5F_ACC_TRUNC   2u
#define H5S_SCALAR      0
#define H5S_SIMPLE      1
#define H5T_COMPOUND    6
#define H5T_STRING      3
#define H5T_VARIABLE    ((size_t)-1)
#define H5T_STR_NULLTERM 0
#define H5T_CSET_ASCII  0
#define H5P_DATASET_CREATE ((hid_t)0)
#define H5P_LINK_CREATE    ((hid_t)0)
#define H5P_GROUP_CREATE   ((hid_t)0)
#define H5E_DEFAULT        ((hid_t)0)
#define H5O_TYPE_GROUP     0
#define H5O_TYPE_DATASET   1
#define H5_ITER_INC        0
#define H5_INDEX_NAME      0

/* native type handles: distinct small integers, never dereferenced */
#define H5T_NATIVE_CHAR    ((hid_t)101)
#define H5T_NATIVE_UCHAR   ((hid_t)102)
#define H5T_NATIVE_SHORT   ((hid_t)103)
#define H5T_NATIVE_USHORT  ((hid_t)104)
#define H5T_NATIVE_INT     ((hid_t)105)
#define H5T_NATIVE_UINT    ((hid_t)106)
#define H5T_NATIVE_LONG    ((hid_t)107)
#define H5T_NATIVE_ULONG   ((hid_t)108)
#define H5T_NATIVE_LLONG   ((hid_t)109)
#define H5T_NATIVE_ULLONG  ((hid_t)110)
#define H5T_NATIVE_FLOAT   ((hid_t)111)
#define H5T_NATIVE_DOUBLE  ((hid_t)112)
#define H5T_NATIVE_LDOUBLE ((hid_t)113)
#define H5T_NATIVE_HBOOL   ((hid_t)114)
#define H5T_NATIVE_INT32   ((hid_t)115)
#define H5T_NATIVE_UINT32  ((hid_t)116)
#define H5T_NATIVE_INT64   ((hid_t)117)
#define H5T_NATIVE_UINT64  ((hid_t)118)
#define H5T_NATIVE_INT8    ((hid_t)119)
#define H5T_NATIVE_UINT8   ((hid_t)120)
#define H5T_C_S1           ((hid_t)121)
#define H5T_STD_I32LE      ((hid_t)122)
#define H5T_IEEE_F64LE     ((hid_t)123)

/* every call fails: the harness never performs QDF I/O */
#define QHG_H5_NOOP_HID(name)  static inline hid_t  name(...) { return (hid_t)-1; }
#define QHG_H5_NOOP_ERR(name)  static inline herr_t name(...) { return -1; }

QHG_H5_NOOP_HID(H5Fcreate)  QHG_H5_NOOP_HID(H5Fopen)   QHG_H5_NOOP_ERR(H5Fclose)
QHG_H5_NOOP_HID(H5Gcreate)  QHG_H5_NOOP_HID(H5Gcreate2) QHG_H5_NOOP_HID(H5Gopen)
QHG_H5_NOOP_HID(H5Gopen2)   QHG_H5_NOOP_ERR(H5Gclose)
QHG_H5_NOOP_HID(H5Screate)  QHG_H5_NOOP_HID(H5Screate_simple) QHG_H5_NOOP_ERR(H5Sclose)
QHG_H5_NOOP_ERR(H5Sselect_hyperslab) QHG_H5_NOOP_ERR(H5Sget_simple_extent_dims)
QHG_H5_NOOP_ERR(H5Sget_simple_extent_ndims) QHG_H5_NOOP_ERR(H5Sselect_all)
QHG_H5_NOOP_HID(H5Dcreate)  QHG_H5_NOOP_HID(H5Dcreate2) QHG_H5_NOOP_HID(H5Dopen)
QHG_H5_NOOP_HID(H5Dopen2)   QHG_H5_NOOP_ERR(H5Dclose)  QHG_H5_NOOP_ERR(H5Dread)
QHG_H5_NOOP_ERR(H5Dwrite)   QHG_H5_NOOP_HID(H5Dget_space) QHG_H5_NOOP_HID(H5Dget_type)
QHG_H5_NOOP_HID(H5Tcreate)  QHG_H5_NOOP_HID(H5Tcopy)   QHG_H5_NOOP_ERR(H5Tclose)
QHG_H5_NOOP_ERR(H5Tinsert)  QHG_H5_NOOP_ERR(H5Tset_size) QHG_H5_NOOP_ERR(H5Tequal)
QHG_H5_NOOP_ERR(H5Tget_class) QHG_H5_NOOP_ERR(H5Tget_size) QHG_H5_NOOP_ERR(H5Tset_strpad)
QHG_H5_NOOP_ERR(H5Tget_nmembers) QHG_H5_NOOP_ERR(H5Tis_variable_str)
QHG_H5_NOOP_HID(H5Acreate)  QHG_H5_NOOP_HID(H5Acreate2) QHG_H5_NOOP_HID(H5Aopen)
QHG_H5_NOOP_HID(H5Aopen_name) QHG_H5_NOOP_ERR(H5Aclose) QHG_H5_NOOP_ERR(H5Aread)
QHG_H5_NOOP_ERR(H5Awrite)   QHG_H5_NOOP_HID(H5Aget_type) QHG_H5_NOOP_HID(H5Aget_space)
QHG_H5_NOOP_ERR(H5Aexists)  QHG_H5_NOOP_ERR(H5Lexists) QHG_H5_NOOP_ERR(H5Literate)
QHG_H5_NOOP_HID(H5Pcreate)  QHG_H5_NOOP_ERR(H5Pclose)  QHG_H5_NOOP_ERR(H5Pset_chunk)
QHG_H5_NOOP_ERR(H5Pset_deflate) QHG_H5_NOOP_ERR(H5Eset_auto) QHG_H5_NOOP_ERR(H5Eset_auto2)
QHG_H5_NOOP_ERR(H5Oget_info) QHG_H5_NOOP_ERR(H5Oget_info_by_name) QHG_H5_NOOP_ERR(H5Gget_info)
QHG_H5_NOOP_ERR(H5Dvlen_reclaim)

#undef QHG_H5_NOOP_HID
#undef QHG_H5_NOOP_ERR

#endif
