// wm_pio.cuh -- host side of the snapshot and output files (common/paraio.f90, one rank).
//
// A file pair <name>.json + <name>.raw: the raw file holds every attribute and dataset back to
// back at a running displacement (utils/iocore/mpiio.f90 write_atomic / write_collective advance
// it by the bytes written); the JSON document describes each one with the keys that
// utils/iocore/jsonio.f90 put_metadata_ik writes (datatype, offset, size, ndim, shape,
// description, plus data for attributes), printed in json-fortran's layout.
#pragma once
#include <stdint.h>
#include <stdio.h>

#include <string>
#include <utility>
#include <vector>

#include "wm_internal.cuh"

namespace wmpio {

// ------------------------------------------------------------------ JSON values
struct JVal {
    enum Kind { NUL, BOOL, INT, REAL, STR, OBJ, ARR } k = NUL;
    long long i = 0;
    double d = 0.0;
    std::string s;
    std::vector<std::pair<std::string, JVal>> obj;
    std::vector<JVal> arr;

    static JVal integer(long long v)
    {
        JVal j;
        j.k = INT;
        j.i = v;
        return j;
    }
    static JVal real(double v)
    {
        JVal j;
        j.k = REAL;
        j.d = v;
        return j;
    }
    static JVal str(const std::string &v)
    {
        JVal j;
        j.k = STR;
        j.s = v;
        return j;
    }
    static JVal object()
    {
        JVal j;
        j.k = OBJ;
        return j;
    }
    static JVal array()
    {
        JVal j;
        j.k = ARR;
        return j;
    }
    JVal &add(const std::string &name, JVal v);  // append to an object, returns the new member
    const JVal *get(const std::string &name) const;
    long long as_int() const { return k == INT ? i : (long long)d; }
    double as_real() const { return k == REAL ? d : (double)i; }
};

std::string fortran_real(double v);         // json-fortran's '(ss,E27.17E4)' + compact_real_string
std::string dumps(const JVal &root);         // json%print layout
bool parse(const std::string &text, JVal &out);

// ------------------------------------------------------------------ file pair
class Writer {
  public:
    // opens dir+name.raw for writing; the JSON is written by close()
    int open(const std::string &dir, const std::string &name);
    int attr_i4(const char *name, int v);
    int attr_i8(const char *name, long long v);
    int attr_f8(const char *name, double v);
    int attr_f8v(const char *name, const double *v, int n);
    // a dataset entry at the current displacement; its bytes follow through write()
    int dataset(const char *name, const char *dt, const std::vector<long long> &shape, const char *desc);
    int write(const void *p, size_t bytes);
    int close();  // writes the JSON, closes the raw file
    ~Writer();

  private:
    JVal root_;
    JVal *att_ = nullptr, *ds_ = nullptr;
    FILE *raw_ = nullptr;
    long long disp_ = 0;
    long long end_ = 0;  // where the last entry's bytes end: close() checks they were all written
    std::string json_path_;
    JVal &entry(JVal *&group, const char *grp, const char *name, const char *dt, const std::vector<long long> &shape,
                long long elem, const char *desc);
};

// A dataset of the file pair read back: byte offset and Fortran shape.
struct Entry {
    std::string datatype;
    long long offset = 0, size = 0;
    std::vector<long long> shape;
};

class Reader {
  public:
    int open(const std::string &dir, const std::string &name);
    int find(const char *group, const char *name, Entry &e) const;
    int read(const Entry &e, void *dst, size_t bytes) const;
    int read_i4(const char *name, int &v) const;
    int read_f8(const char *name, double *v, int n) const;
    ~Reader();

  private:
    JVal root_;
    FILE *raw_ = nullptr;
};

// The module state of paraio__init (paraio.f90:37-72).
struct Params {
    int ndim = 0, np = 0, nsp = 0, nxgs = 0, nxge = 0, nygs = 0, nyge = 0, nys = 0, nye = 0, nproc = 1;
    double delx = 0, delt = 0, c = 0;
    double q[WM_MAX_SP] = {0}, r[WM_MAX_SP] = {0};
    std::string dir;
};

// The attributes every paraio file starts with: dummy_attribute, it, [extra i4 ...], then
// put_metadata (paraio.f90:947-1002).
int write_head(Writer &w, const Params &P, int it, const std::vector<std::pair<const char *, int>> &extra);

// Copy `bytes` from device memory into the file through a pinned double buffer, so the next
// chunk's copy overlaps the write of the previous one.
int write_from_device(Writer &w, const void *dev, size_t bytes, cudaStream_t st);

// nrows rows of the file, each `dst_row` bytes: the first `src_row` bytes of device row r (device
// rows `src_row` bytes apart), then zeros.  Used for up(ndim, np, ...) from packed rows.
int write_rows_from_device(Writer &w, const void *dev, size_t src_row, size_t dst_row, long long nrows, cudaStream_t st);

}  // namespace wmpio
