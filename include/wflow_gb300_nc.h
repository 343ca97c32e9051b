/*
 * wflow_gb300_nc.h -- netCDF classic-format files for the step library's inputs and states.
 *
 * Wflow reads its static maps, forcing and initial states from netCDF files and writes its
 * states back (Wflow/src/io.jl:65-227, 432-899; utils.jl:161-213; states.jl). This is a
 * self-contained reader and writer of the netCDF classic binary formats (CDF-1 classic, CDF-2
 * 64-bit offset, CDF-5 64-bit data) following the published netCDF file-format specification:
 * big-endian header of dimensions, attributes and variables, fixed-size variables stored
 * contiguously, record variables interleaved record by record. netCDF-4 (HDF5) files are not
 * read: convert them with `nccopy -k cdf5` (or `-k classic`) first.
 *
 * Values cross the boundary as doubles: wf_nc_get converts from the stored type and, with
 * decode set, applies the CF conventions NCDatasets applies when Wflow reads a variable
 * (_FillValue / missing_value -> NaN, then scale_factor and add_offset); wf_nc_put converts
 * to the stored type (integers rounded to nearest, out-of-range values rejected; NaN written
 * as the variable's _FillValue, or the type's default fill value).
 */
#ifndef WFLOW_GB300_NC_H
#define WFLOW_GB300_NC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* netCDF external types (nc_type) */
typedef enum WfNcType {
    WF_NC_BYTE = 1,
    WF_NC_CHAR = 2,
    WF_NC_SHORT = 3,
    WF_NC_INT = 4,
    WF_NC_FLOAT = 5,
    WF_NC_DOUBLE = 6,
    WF_NC_UBYTE = 7, /* CDF-5 only from here */
    WF_NC_USHORT = 8,
    WF_NC_UINT = 9,
    WF_NC_INT64 = 10,
    WF_NC_UINT64 = 11
} WfNcType;

#define WF_NC_GLOBAL (-1) /* varid of the global attributes */

typedef struct WfNcFile WfNcFile;

/* ---- reading --------------------------------------------------------------------------- */
/* Open an existing file read-only. Returns 0 or a negative WfStatus (the message is in
 * wf_nc_last_error(NULL) when *out is NULL). */
int32_t wf_nc_open(const char* path, WfNcFile** out);
void wf_nc_close(WfNcFile* f);
const char* wf_nc_last_error(const WfNcFile* f);
/* 1 (classic), 2 (64-bit offset) or 5 (64-bit data) */
int32_t wf_nc_format(const WfNcFile* f);
int64_t wf_nc_numrecs(const WfNcFile* f);
int32_t wf_nc_ndims(const WfNcFile* f);
int32_t wf_nc_nvars(const WfNcFile* f);
/* Dimension i: name (NUL-terminated, truncated to cap), length (the current number of records
 * for the record dimension), is_record. */
int32_t wf_nc_dim(const WfNcFile* f, int32_t i, char* name, int32_t cap, int64_t* len, int32_t* is_record);
/* Variable i: name, type, number of dimensions and their ids (dimids has room for 16). */
int32_t wf_nc_var(const WfNcFile* f, int32_t i, char* name, int32_t cap, int32_t* type, int32_t* ndims,
                  int32_t* dimids);
/* Id of a variable by name, or -1. */
int32_t wf_nc_varid(const WfNcFile* f, const char* name);
/* Number of attributes of variable varid (WF_NC_GLOBAL for the file) and the name of the i-th. */
int32_t wf_nc_natts(const WfNcFile* f, int32_t varid);
int32_t wf_nc_att_name(const WfNcFile* f, int32_t varid, int32_t i, char* name, int32_t cap);
/* Attribute `name` of variable varid (WF_NC_GLOBAL for the file): type and number of values;
 * returns -1 (WF_ERR_INVALID) when absent. */
int32_t wf_nc_att(const WfNcFile* f, int32_t varid, const char* name, int32_t* type, int64_t* n);
/* Its values as doubles (numeric attributes) or its text (char attributes, NUL-terminated). */
int32_t wf_nc_att_get(const WfNcFile* f, int32_t varid, const char* name, double* dst, int64_t cap);
int32_t wf_nc_att_text(const WfNcFile* f, int32_t varid, const char* name, char* dst, int64_t cap);
/* Hyperslab [start, start + count) of variable varid (C order, record dimension first) as
 * doubles; decode != 0 applies the CF decoding described above. */
int32_t wf_nc_get(WfNcFile* f, int32_t varid, const int64_t* start, const int64_t* count, double* dst,
                  int32_t decode);

/* ---- writing --------------------------------------------------------------------------- */
/* Create (overwrite) a file in define mode; format 1, 2 or 5. */
int32_t wf_nc_create(const char* path, int32_t format, WfNcFile** out);
/* A dimension of length len (0 = the record dimension, at most one); returns its id >= 0. */
int32_t wf_nc_def_dim(WfNcFile* f, const char* name, int64_t len);
/* A variable; returns its id >= 0. */
int32_t wf_nc_def_var(WfNcFile* f, const char* name, int32_t type, int32_t ndims, const int32_t* dimids);
int32_t wf_nc_put_att_text(WfNcFile* f, int32_t varid, const char* name, const char* text);
int32_t wf_nc_put_att(WfNcFile* f, int32_t varid, const char* name, int32_t type, const double* values, int64_t n);
/* Leave define mode: lay out the data, write the header and the fill values. */
int32_t wf_nc_enddef(WfNcFile* f);
/* Write a hyperslab from doubles (data mode); writing past the last record adds records. */
int32_t wf_nc_put(WfNcFile* f, int32_t varid, const int64_t* start, const int64_t* count, const double* src);

#ifdef __cplusplus
}
#endif

#endif /* WFLOW_GB300_NC_H */
