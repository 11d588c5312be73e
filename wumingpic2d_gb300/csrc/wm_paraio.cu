// wm_paraio.cu -- the snapshot and output files of common/paraio.f90 (one rank).
//
//   host layer    JSON printer / parser and the raw-file writer (wm_pio.cuh); the drop-in
//                 procedures wm_paraio_* on host arrays, argument for argument those of the
//                 Fortran module (paraio__init/_output/_input/_param/_mom/_ptcl/_orb).
//   device layer  kernels that put the resident state into file order on the GPU: moments
//                 divided by the density and cell-centred fields (paraio__mom), the interior
//                 fields and the ordered compaction of active particles or tracers
//                 (write_particle / get_particle_count); the host only streams the bytes to disk.
#include <errno.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include "wm_launch.cuh"
#include "wm_pio.cuh"

namespace wmpio {

// ======================================================================= JSON
JVal &JVal::add(const std::string &name, JVal v)
{
    obj.emplace_back(name, std::move(v));
    return obj.back().second;
}

const JVal *JVal::get(const std::string &name) const
{
    for (const auto &m : obj)
        if (m.first == name) return &m.second;
    return nullptr;
}

// json-fortran writes a real(8) with '(ss,E27.17E4)' -- 0.d1...d17E+eeee, correctly rounded
// to 17 digits -- and compact_real_string (json_string_utilities.F90:266-334) then drops the
// trailing zeros of the digits (keeping one) and the leading zeros of the exponent.
std::string fortran_real(double v)
{
    const bool neg = signbit(v);
    const double a = fabs(v);
    char digits[32];
    int exp10 = 0;
    if (a == 0.0) {
        memset(digits, '0', 17);
        digits[17] = 0;
    } else {
        char buf[64];
        snprintf(buf, sizeof buf, "%.16e", a);  // d.dddddddddddddddde+XX
        digits[0] = buf[0];
        memcpy(digits + 1, buf + 2, 16);
        digits[17] = 0;
        exp10 = atoi(strchr(buf, 'e') + 1) + 1;
    }
    int n = 17;
    while (n > 1 && digits[n - 1] == '0') --n;
    std::string s = neg ? "-0." : "0.";
    s.append(digits, n);
    s += exp10 < 0 ? "E-" : "E+";
    s += std::to_string(exp10 < 0 ? -exp10 : exp10);
    return s;
}

static void quote(std::string &o, const std::string &s)
{
    o += '"';
    for (char ch : s) {
        switch (ch) {
        case '"': o += "\\\""; break;
        case '\\': o += "\\\\"; break;
        case '\n': o += "\\n"; break;
        case '\r': o += "\\r"; break;
        case '\t': o += "\\t"; break;
        case '\b': o += "\\b"; break;
        case '\f': o += "\\f"; break;
        default: o += ch;
        }
    }
    o += '"';
}

static void emit(const JVal &v, int ind, const std::string &prefix, std::vector<std::string> &lines)
{
    const std::string pad(2 * ind, ' ');
    std::string line = pad + prefix;
    switch (v.k) {
    case JVal::OBJ:
        lines.push_back(line + "{");
        for (size_t n = 0; n < v.obj.size(); ++n) {
            std::string key;
            quote(key, v.obj[n].first);
            emit(v.obj[n].second, ind + 1, key + ": ", lines);
            if (n + 1 < v.obj.size()) lines.back() += ",";
        }
        lines.push_back(pad + "}");
        return;
    case JVal::ARR:
        lines.push_back(line + "[");
        for (size_t n = 0; n < v.arr.size(); ++n) {
            emit(v.arr[n], ind + 1, "", lines);
            if (n + 1 < v.arr.size()) lines.back() += ",";
        }
        lines.push_back(pad + "]");
        return;
    case JVal::INT: line += std::to_string(v.i); break;
    case JVal::REAL: line += fortran_real(v.d); break;
    case JVal::STR: quote(line, v.s); break;
    case JVal::BOOL: line += v.i ? "true" : "false"; break;
    default: line += "null";
    }
    lines.push_back(line);
}

std::string dumps(const JVal &root)
{
    std::vector<std::string> lines;
    emit(root, 0, "", lines);
    std::string out;
    for (const auto &l : lines) {
        out += l;
        out += '\n';
    }
    return out;
}

namespace {
struct Parser {
    const char *p, *end;
    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    bool lit(const char *w)
    {
        const size_t n = strlen(w);
        if ((size_t)(end - p) < n || strncmp(p, w, n) != 0) return false;
        p += n;
        return true;
    }
    bool str(std::string &s)
    {
        if (p >= end || *p != '"') return false;
        ++p;
        s.clear();
        while (p < end && *p != '"') {
            char ch = *p++;
            if (ch == '\\') {
                if (p >= end) return false;
                const char e = *p++;
                switch (e) {
                case 'n': ch = '\n'; break;
                case 'r': ch = '\r'; break;
                case 't': ch = '\t'; break;
                case 'b': ch = '\b'; break;
                case 'f': ch = '\f'; break;
                case 'u':  // keep the escape as text; the files here are ASCII
                    s += "\\u";
                    continue;
                default: ch = e;
                }
            }
            s += ch;
        }
        if (p >= end) return false;
        ++p;
        return true;
    }
    bool value(JVal &v, int depth)
    {
        if (depth > 64) return false;
        ws();
        if (p >= end) return false;
        if (*p == '{') {
            ++p;
            v = JVal::object();
            ws();
            if (p < end && *p == '}') return ++p, true;
            for (;;) {
                ws();
                std::string key;
                if (!str(key)) return false;
                ws();
                if (p >= end || *p != ':') return false;
                ++p;
                JVal m;
                if (!value(m, depth + 1)) return false;
                v.add(key, std::move(m));
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == '}') return ++p, true;
                return false;
            }
        }
        if (*p == '[') {
            ++p;
            v = JVal::array();
            ws();
            if (p < end && *p == ']') return ++p, true;
            for (;;) {
                JVal m;
                if (!value(m, depth + 1)) return false;
                v.arr.push_back(std::move(m));
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == ']') return ++p, true;
                return false;
            }
        }
        if (*p == '"') {
            v.k = JVal::STR;
            return str(v.s);
        }
        if (lit("true")) {
            v.k = JVal::BOOL;
            v.i = 1;
            return true;
        }
        if (lit("false")) {
            v.k = JVal::BOOL;
            v.i = 0;
            return true;
        }
        if (lit("null")) {
            v.k = JVal::NUL;
            return true;
        }
        const char *q = p;
        bool real = false;
        while (q < end && (isdigit((unsigned char)*q) || *q == '-' || *q == '+' || *q == '.' || *q == 'e' || *q == 'E' ||
                           *q == 'd' || *q == 'D')) {
            if (*q == '.' || *q == 'e' || *q == 'E' || *q == 'd' || *q == 'D') real = true;
            ++q;
        }
        if (q == p) return false;
        std::string num(p, q);
        for (char &ch : num)
            if (ch == 'd' || ch == 'D') ch = 'E';
        errno = 0;
        char *stop = nullptr;
        if (real) {
            v.k = JVal::REAL;
            v.d = strtod(num.c_str(), &stop);
        } else {
            v.k = JVal::INT;
            v.i = strtoll(num.c_str(), &stop, 10);
        }
        if (!stop || *stop != 0 || errno == ERANGE) return false;
        p = q;
        return true;
    }
};
}  // namespace

bool parse(const std::string &text, JVal &out)
{
    Parser ps{text.data(), text.data() + text.size()};
    if (!ps.value(out, 0)) return false;
    ps.ws();
    return ps.p == ps.end;
}

// ======================================================================= files
static int endian_flag()
{
    // mpiio.f90:102-109: the bytes (1,0,0,0) read as a 4-byte integer
    const unsigned char b[4] = {1, 0, 0, 0};
    int32_t f;
    memcpy(&f, b, 4);
    return f;
}

Writer::~Writer()
{
    if (raw_) fclose(raw_);
}

int Writer::open(const std::string &dir, const std::string &name)
{
    raw_ = fopen((dir + name + ".raw").c_str(), "wb");
    if (!raw_) return WM_ERR_IO;
    json_path_ = dir + name + ".json";
    root_ = JVal::object();
    root_.obj.reserve(4);  // meta, attribute, dataset: the group pointers below stay valid
    JVal &meta = root_.add("meta", JVal::object());
    meta.add("endian", JVal::integer(endian_flag()));
    meta.add("rawfile", JVal::str(name + ".raw"));
    disp_ = 0;
    return WM_OK;
}

JVal &Writer::entry(JVal *&group, const char *grp, const char *name, const char *dt, const std::vector<long long> &shape,
                    long long elem, const char *desc)
{
    if (!group) group = &root_.add(grp, JVal::object());
    long long n = 1;
    for (long long s : shape) n *= s;
    JVal e = JVal::object();
    e.add("datatype", JVal::str(dt));
    e.add("offset", JVal::integer(disp_));
    e.add("size", JVal::integer(n * elem));
    e.add("ndim", JVal::integer((long long)shape.size()));
    JVal sh = JVal::array();
    for (long long s : shape) sh.arr.push_back(JVal::integer(s));
    e.add("shape", std::move(sh));
    e.add("description", JVal::str(desc));
    end_ = disp_ + n * elem;
    return group->add(name, std::move(e));
}

int Writer::write(const void *p, size_t bytes)
{
    if (!raw_) return WM_ERR_IO;
    if (bytes && fwrite(p, 1, bytes, raw_) != bytes) return WM_ERR_IO;
    disp_ += (long long)bytes;
    return WM_OK;
}

int Writer::attr_i4(const char *name, int v)
{
    JVal &e = entry(att_, "attribute", name, "i4", {1}, 4, "");
    e.add("data", JVal::integer(v));
    const int32_t x = v;
    return write(&x, 4);
}

int Writer::attr_i8(const char *name, long long v)
{
    JVal &e = entry(att_, "attribute", name, "i8", {1}, 8, "");
    e.add("data", JVal::integer(v));
    const int64_t x = v;
    return write(&x, 8);
}

int Writer::attr_f8(const char *name, double v)
{
    JVal &e = entry(att_, "attribute", name, "f8", {1}, 8, "");
    e.add("data", JVal::real(v));
    return write(&v, 8);
}

int Writer::attr_f8v(const char *name, const double *v, int n)
{
    JVal &e = entry(att_, "attribute", name, "f8", {(long long)n}, 8, "");
    JVal d = JVal::array();
    for (int k = 0; k < n; ++k) d.arr.push_back(JVal::real(v[k]));
    e.add("data", std::move(d));
    return write(v, sizeof(double) * n);
}

int Writer::dataset(const char *name, const char *dt, const std::vector<long long> &shape, const char *desc)
{
    const long long elem = (dt[1] == '8') ? 8 : 4;
    entry(ds_, "dataset", name, dt, shape, elem, desc);
    return WM_OK;
}

int Writer::close()
{
    if (!raw_) return WM_ERR_IO;
    const bool ok = fclose(raw_) == 0 && disp_ == end_;
    raw_ = nullptr;
    if (!ok) return WM_ERR_IO;
    FILE *f = fopen(json_path_.c_str(), "w");
    if (!f) return WM_ERR_IO;
    const std::string text = dumps(root_);
    const bool wr = fwrite(text.data(), 1, text.size(), f) == text.size();
    return (fclose(f) == 0 && wr) ? WM_OK : WM_ERR_IO;
}

Reader::~Reader()
{
    if (raw_) fclose(raw_);
}

int Reader::open(const std::string &dir, const std::string &name)
{
    FILE *f = fopen((dir + name + ".json").c_str(), "rb");
    if (!f) return WM_ERR_IO;
    std::string text;
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    fclose(f);
    if (!parse(text, root_) || root_.k != JVal::OBJ) return WM_ERR_IO;
    raw_ = fopen((dir + name + ".raw").c_str(), "rb");  // paraio__input opens filename.raw
    return raw_ ? WM_OK : WM_ERR_IO;
}

int Reader::find(const char *group, const char *name, Entry &e) const
{
    const JVal *g = root_.get(group);
    const JVal *v = g ? g->get(name) : nullptr;
    if (!v || v->k != JVal::OBJ) return WM_ERR_IO;
    const JVal *dt = v->get("datatype"), *off = v->get("offset"), *sh = v->get("shape"), *sz = v->get("size");
    if (!dt || !off || !sh || sh->k != JVal::ARR) return WM_ERR_IO;
    e.datatype = dt->s;
    e.offset = off->as_int();
    e.shape.clear();
    for (const auto &x : sh->arr) e.shape.push_back(x.as_int());
    e.size = sz ? sz->as_int() : 0;
    return WM_OK;
}

int Reader::read(const Entry &e, void *dst, size_t bytes) const
{
    if (!raw_ || fseeko(raw_, (off_t)e.offset, SEEK_SET) != 0) return WM_ERR_IO;
    return fread(dst, 1, bytes, raw_) == bytes ? WM_OK : WM_ERR_IO;
}

int Reader::read_i4(const char *name, int &v) const
{
    Entry e;
    WM_TRY(find("attribute", name, e));
    if (e.datatype != "i4") return WM_ERR_IO;
    int32_t x;
    WM_TRY(read(e, &x, 4));
    v = x;
    return WM_OK;
}

int Reader::read_f8(const char *name, double *v, int n) const
{
    Entry e;
    WM_TRY(find("attribute", name, e));
    long long cnt = 1;
    for (long long s : e.shape) cnt *= s;
    if (e.datatype != "f8" || cnt != n) return WM_ERR_IO;
    return read(e, v, sizeof(double) * n);
}

int write_head(Writer &w, const Params &P, int it, const std::vector<std::pair<const char *, int>> &extra)
{
    WM_TRY(w.attr_i8("dummy_attribute", 8));  // MPI_OFFSET_KIND
    WM_TRY(w.attr_i4("it", it));
    for (const auto &x : extra) WM_TRY(w.attr_i4(x.first, x.second));
    WM_TRY(w.attr_i4("ndim", P.ndim));
    WM_TRY(w.attr_i4("np", P.np));
    WM_TRY(w.attr_i4("nxgs", P.nxgs));
    WM_TRY(w.attr_i4("nxge", P.nxge));
    WM_TRY(w.attr_i4("nygs", P.nygs));
    WM_TRY(w.attr_i4("nyge", P.nyge));
    WM_TRY(w.attr_i4("nsp", P.nsp));
    WM_TRY(w.attr_i4("nproc", P.nproc));
    WM_TRY(w.attr_f8("delx", P.delx));
    WM_TRY(w.attr_f8("delt", P.delt));
    WM_TRY(w.attr_f8("c", P.c));
    WM_TRY(w.attr_f8v("r", P.r, P.nsp));
    return w.attr_f8v("q", P.q, P.nsp);
}

namespace {
// Pinned double buffer for device -> file streaming, kept for the life of the process.
struct Bounce {
    static constexpr size_t CHUNK = 64u << 20;
    void *buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int ensure()
    {
        for (int b = 0; b < 2; ++b) {
            if (!buf[b]) WM_CUDA(cudaHostAlloc(&buf[b], CHUNK, cudaHostAllocPortable));
            if (!ev[b]) WM_CUDA(cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming));
        }
        return WM_OK;
    }
};
Bounce g_bounce;
}  // namespace

int write_from_device(Writer &w, const void *dev, size_t bytes, cudaStream_t st)
{
    if (bytes == 0) return WM_OK;
    WM_TRY(g_bounce.ensure());
    const size_t C = Bounce::CHUNK;
    const size_t nchunk = (bytes + C - 1) / C;
    for (size_t c = 0; c <= nchunk; ++c) {
        if (c < nchunk) {  // chunk c into buffer c%2 (its previous contents were written at step c-1)
            const size_t n = std::min(C, bytes - c * C);
            WM_CUDA(cudaMemcpyAsync(g_bounce.buf[c & 1], (const char *)dev + c * C, n, cudaMemcpyDeviceToHost, st));
            WM_CUDA(cudaEventRecord(g_bounce.ev[c & 1], st));
        }
        if (c > 0) {  // write chunk c-1 while chunk c is in flight
            const size_t p = c - 1, n = std::min(C, bytes - p * C);
            WM_CUDA(cudaEventSynchronize(g_bounce.ev[p & 1]));
            WM_TRY(w.write(g_bounce.buf[p & 1], n));
        }
    }
    return WM_OK;
}

int write_rows_from_device(Writer &w, const void *dev, size_t src_row, size_t dst_row, long long nrows, cudaStream_t st)
{
    if (src_row > dst_row) return WM_ERR_BAD_ARG;
    WM_TRY(g_bounce.ensure());
    const size_t C = Bounce::CHUNK;
    if (dst_row > C) {  // rows longer than a buffer: the device part in pieces, then the zeros
        static const std::vector<char> zeros(1 << 20, 0);
        for (long long r = 0; r < nrows; ++r) {
            WM_TRY(write_from_device(w, (const char *)dev + r * src_row, src_row, st));
            for (size_t z = dst_row - src_row; z > 0;) {
                const size_t n = std::min(z, zeros.size());
                WM_TRY(w.write(zeros.data(), n));
                z -= n;
            }
        }
        return WM_OK;
    }
    // several rows per buffer: pitched copies leave the row tails untouched, so zero them once
    for (int b = 0; b < 2; ++b) memset(g_bounce.buf[b], 0, C);
    const long long per = (long long)(C / dst_row);
    const long long nchunk = (nrows + per - 1) / per;
    for (long long c = 0; c <= nchunk; ++c) {
        if (c < nchunk) {
            const long long r0 = c * per, k = std::min(per, nrows - r0);
            WM_CUDA(cudaMemcpy2DAsync(g_bounce.buf[c & 1], dst_row, (const char *)dev + r0 * src_row, src_row, src_row, (size_t)k,
                                      cudaMemcpyDeviceToHost, st));
            WM_CUDA(cudaEventRecord(g_bounce.ev[c & 1], st));
        }
        if (c > 0) {
            const long long p = c - 1, k = std::min(per, nrows - p * per);
            WM_CUDA(cudaEventSynchronize(g_bounce.ev[p & 1]));
            WM_TRY(w.write(g_bounce.buf[p & 1], (size_t)k * dst_row));
        }
    }
    return WM_OK;
}

}  // namespace wmpio

// ============================================================== device kernels
namespace {

// paraio.f90:626-671 in file order: den(nx,ny,nsp), vel(3,nx,ny,nsp) = mom(2:4)/mom(1),
// temp(3,nx,ny,nsp) = mom(5:7)/mom(1), then the cell-centred fields tmp(6,nx,ny) with the
// Bz average as written there (uf(3,i+1,j) twice, uf(3,i,j+1) not at all).
__global__ void k_mom_file(WmGeom g, const double *__restrict__ mom, FView<6, false> uf, double *__restrict__ out)
{
    const long long ncell = (long long)g.nx * g.ny;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= ncell * g.nsp) return;
    const int ci = (int)(t % g.nx), cj = (int)((t / g.nx) % g.ny), isp = (int)(t / ncell);
    // mom(7, nxgs-1:nxge+1, nys-1:nye+1, nsp), component fastest
    const double *m = mom + 7 * ((ci + 1) + (long long)(g.nx + 2) * ((cj + 1) + (long long)(g.ny + 2) * isp));
    const double den = m[0];
    out[t] = den;
    double *vel = out + ncell * g.nsp, *temp = vel + 3 * ncell * g.nsp;
    for (int k = 0; k < 3; ++k) {
        vel[3 * t + k] = m[1 + k] / den;
        temp[3 * t + k] = m[4 + k] / den;
    }
    if (isp == 0) {
        double *cf = temp + 3 * ncell * g.nsp + 6 * (ci + (long long)g.nx * cj);
        const int ix = ci + 2, iy = cj + 2;
        cf[0] = (uf(0, ix, iy) + uf(0, ix, iy + 1)) / 2;
        cf[1] = (uf(1, ix, iy) + uf(1, ix + 1, iy)) / 2;
        cf[2] = (uf(2, ix, iy) + uf(2, ix + 1, iy) + uf(2, ix + 1, iy) + uf(2, ix + 1, iy + 1)) / 4;
        cf[3] = (uf(3, ix, iy) + uf(3, ix + 1, iy)) / 2;
        cf[4] = (uf(4, ix, iy) + uf(4, ix, iy + 1)) / 2;
        cf[5] = uf(5, ix, iy);
    }
}

// uf(1:6, nxgs:nxge, nys:nye), component fastest (write_particle, paraio.f90:808-823)
__global__ void k_uf_interior(WmGeom g, FView<6, false> uf, double *__restrict__ out)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)g.nx * g.ny) return;
    const int ci = (int)(t % g.nx), cj = (int)(t / g.nx);
    for (int k = 0; k < 6; ++k) out[6 * t + k] = uf(k, ci + 2, cj + 2);
}

// get_particle_count (paraio.f90:854-942): particles of a row that go to the file -- all active
// ones (mode 0) or those whose id, the bits of the sixth double, is positive (mode 1).
__device__ __forceinline__ bool selected(const double *a, int mode)
{
    return mode == 0 || __double_as_longlong(a[5]) > 0;
}

constexpr int ROW_THREADS = 256;

__global__ void __launch_bounds__(ROW_THREADS) k_row_count(const double *__restrict__ stage, int pitch, const int *__restrict__ np2,
                                                           int mode, long long *__restrict__ cnt)
{
    const int row = blockIdx.x, n = np2[row];
    int c = 0;
    for (int s = threadIdx.x; s < n; s += blockDim.x) c += selected(stage + 6 * ((long long)row * pitch + s), mode);
    __shared__ int red[ROW_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < ROW_THREADS / 32; ++w) t += red[w];
        cnt[row] = t;
    }
}

// Ordered compaction of one row: the selected particles keep their slot order (the Fortran
// packs j = nys..nye, i = 1..np2(j) per species).
__global__ void __launch_bounds__(ROW_THREADS) k_row_compact(const double *__restrict__ stage, int pitch, const int *__restrict__ np2,
                                                             int mode, const long long *__restrict__ off, double *__restrict__ out)
{
    const int row = blockIdx.x, n = np2[row];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __shared__ int wsum[ROW_THREADS / 32];
    long long base = off[row];
    for (int s0 = 0; s0 < n; s0 += ROW_THREADS) {
        const int s = s0 + threadIdx.x;
        const double *a = stage + 6 * ((long long)row * pitch + s);
        const bool sel = s < n && selected(a, mode);
        const unsigned m = __ballot_sync(0xffffffffu, sel);
        if (lane == 0) wsum[w] = __popc(m);
        __syncthreads();
        int before = 0, total = 0;
        for (int k = 0; k < ROW_THREADS / 32; ++k) {
            before += (k < w) ? wsum[k] : 0;
            total += wsum[k];
        }
        if (sel) {
            double *d = out + 6 * (base + before + __popc(m & ((1u << lane) - 1)));
            for (int k = 0; k < 6; ++k) d[k] = a[k];
        }
        base += total;
        __syncthreads();
    }
}

}  // namespace

int wm_launch_mom_file(const WmGeom &g, const double *mom, FView<6, false> uf, double *out, cudaStream_t st)
{
    const long long n = (long long)g.nx * g.ny * g.nsp;
    k_mom_file<<<wm_div_up(n, 256), 256, 0, st>>>(g, mom, uf, out);
    return wm_check_launch("k_mom_file");
}

int wm_launch_uf_interior(const WmGeom &g, FView<6, false> uf, double *out, cudaStream_t st)
{
    k_uf_interior<<<wm_div_up((long long)g.nx * g.ny, 256), 256, 0, st>>>(g, uf, out);
    return wm_check_launch("k_uf_interior");
}

int wm_launch_row_count(int nrows, const double *stage, int pitch, const int *np2, int mode, long long *cnt, cudaStream_t st)
{
    k_row_count<<<nrows, ROW_THREADS, 0, st>>>(stage, pitch, np2, mode, cnt);
    return wm_check_launch("k_row_count");
}

int wm_launch_row_compact(int nrows, const double *stage, int pitch, const int *np2, int mode, const long long *off, double *out,
                          cudaStream_t st)
{
    k_row_compact<<<nrows, ROW_THREADS, 0, st>>>(stage, pitch, np2, mode, off, out);
    return wm_check_launch("k_row_compact");
}

// ====================================================== drop-in host procedures
namespace {
struct PioModule {
    bool init = false;
    wmpio::Params P;
};
PioModule g_pio;

int ghost_nx() { return g_pio.P.nxge - g_pio.P.nxgs + 5; }
int ghost_ny() { return g_pio.P.nye - g_pio.P.nys + 5; }
int rows() { return g_pio.P.nye - g_pio.P.nys + 1; }

int write_particles_host(const double *up, const double *uf, const int *np2, int it, int mode)
{
    if (!g_pio.init) return WM_ERR_NOT_INIT;
    if (!up || !uf || !np2) return WM_ERR_BAD_ARG;
    const wmpio::Params &P = g_pio.P;
    char name[64];
    snprintf(name, sizeof name, "%07d%s", it, mode == 0 ? "_ptcl" : "_orb");
    wmpio::Writer w;
    WM_TRY(w.open(P.dir, name));
    WM_TRY(wmpio::write_head(w, P, it, {}));
    const int nx = P.nxge - P.nxgs + 1, ny = P.nyge - P.nygs + 1, nyl = rows(), gx = ghost_nx();
    WM_TRY(w.dataset("uf", "f8", {6, nx, ny}, "electromagnetic field"));
    std::vector<double> line(6 * (size_t)nx);
    for (int j = 0; j < nyl; ++j) {
        memcpy(line.data(), uf + 6 * ((size_t)2 + (size_t)gx * (j + 2)), sizeof(double) * 6 * nx);
        WM_TRY(w.write(line.data(), sizeof(double) * line.size()));
    }
    for (int isp = 0; isp < P.nsp; ++isp) {
        long long npg = 0;
        for (int j = 0; j < nyl; ++j)
            for (int i = 0; i < np2[j + nyl * isp]; ++i) {
                const double *a = up + (size_t)P.ndim * (i + (size_t)P.np * (j + (size_t)nyl * isp));
                int64_t pid;
                memcpy(&pid, a + P.ndim - 1, 8);
                npg += (mode == 0 || pid > 0);
            }
        char ds[16], desc[64];
        snprintf(ds, sizeof ds, "up%02d", isp + 1);
        snprintf(desc, sizeof desc, "particle species #%02d", isp + 1);
        WM_TRY(w.dataset(ds, "f8", {P.ndim, npg}, desc));
        for (int j = 0; j < nyl; ++j)
            for (int i = 0; i < np2[j + nyl * isp]; ++i) {
                const double *a = up + (size_t)P.ndim * (i + (size_t)P.np * (j + (size_t)nyl * isp));
                int64_t pid;
                memcpy(&pid, a + P.ndim - 1, 8);
                if (mode == 0 || pid > 0) WM_TRY(w.write(a, sizeof(double) * P.ndim));
            }
    }
    return w.close();
}
}  // namespace

extern "C" {

int wm_paraio_init(int ndim, int np, int nsp, int nxgs, int nxge, int nygs, int nyge, int nys, int nye, int nproc, int nrank,
                   double delx, double delt, double c, const double *q, const double *r, const char *dir)
{
    if (nproc != 1 || nrank != 0) return WM_ERR_UNSUPPORTED;  // one rank owns every row
    if (nsp < 1 || nsp > WM_MAX_SP || ndim < 1 || np < 1 || !q || !r || !dir) return WM_ERR_BAD_ARG;
    wmpio::Params &P = g_pio.P;
    P.ndim = ndim;
    P.np = np;
    P.nsp = nsp;
    P.nxgs = nxgs;
    P.nxge = nxge;
    P.nygs = nygs;
    P.nyge = nyge;
    P.nys = nys;
    P.nye = nye;
    P.nproc = nproc;
    P.delx = delx;
    P.delt = delt;
    P.c = c;
    for (int s = 0; s < nsp; ++s) {
        P.q[s] = q[s];
        P.r[s] = r[s];
    }
    P.dir = dir;
    g_pio.init = true;
    return WM_OK;
}

int wm_paraio_finalize(void)
{
    g_pio.init = false;
    return WM_OK;
}

int wm_paraio_output(const double *up, const double *uf, const int *np2, int nxs, int nxe, int it, const char *filename)
{
    if (!g_pio.init) return WM_ERR_NOT_INIT;
    if (!up || !uf || !np2 || !filename) return WM_ERR_BAD_ARG;
    const wmpio::Params &P = g_pio.P;
    wmpio::Writer w;
    WM_TRY(w.open(P.dir, filename));
    WM_TRY(wmpio::write_head(w, P, it, {{"nxs", nxs}, {"nxe", nxe}}));
    const long long nyl = rows();
    WM_TRY(w.dataset("up", "f8", {P.ndim, P.np, nyl, P.nsp, P.nproc}, "particles"));
    WM_TRY(w.write(up, sizeof(double) * (size_t)P.ndim * P.np * nyl * P.nsp));
    WM_TRY(w.dataset("np2", "i4", {nyl, P.nsp, P.nproc}, "number of active particles"));
    WM_TRY(w.write(np2, sizeof(int) * (size_t)nyl * P.nsp));
    WM_TRY(w.dataset("uf", "f8", {6, ghost_nx(), ghost_ny(), P.nproc}, "electromagnetic fields including ghost cells"));
    WM_TRY(w.write(uf, sizeof(double) * 6 * (size_t)ghost_nx() * ghost_ny()));
    return w.close();
}

int wm_paraio_input(double *up, double *uf, int *np2, int *nxs, int *nxe, int *it, const char *filename)
{
    if (!g_pio.init) return WM_ERR_NOT_INIT;
    if (!up || !uf || !np2 || !nxs || !nxe || !it || !filename) return WM_ERR_BAD_ARG;
    wmpio::Params &P = g_pio.P;
    wmpio::Reader rd;
    WM_TRY(rd.open(P.dir, filename));
    int v[8];
    WM_TRY(rd.read_i4("it", *it));
    WM_TRY(rd.read_i4("nxs", *nxs));
    WM_TRY(rd.read_i4("nxe", *nxe));
    const char *names[8] = {"ndim", "np", "nxgs", "nxge", "nygs", "nyge", "nsp", "nproc"};
    for (int k = 0; k < 8; ++k) WM_TRY(rd.read_i4(names[k], v[k]));
    if (v[2] != P.nxgs || v[3] != P.nxge || v[4] != P.nygs || v[5] != P.nyge || v[1] != P.np || v[6] != P.nsp ||
        v[7] != P.nproc)
        return WM_ERR_IO;  // paraio.f90:329-340 stops: invalid input parameters
    // paraio.f90:317-327 reads delx, delt, c, r, q into the module variables
    WM_TRY(rd.read_f8("delx", &P.delx, 1));
    WM_TRY(rd.read_f8("delt", &P.delt, 1));
    WM_TRY(rd.read_f8("c", &P.c, 1));
    WM_TRY(rd.read_f8("r", P.r, P.nsp));
    WM_TRY(rd.read_f8("q", P.q, P.nsp));
    const long long nyl = rows();
    wmpio::Entry e;
    WM_TRY(rd.find("dataset", "up", e));
    if (e.shape != std::vector<long long>{P.ndim, P.np, nyl, P.nsp, P.nproc}) return WM_ERR_IO;
    WM_TRY(rd.read(e, up, sizeof(double) * (size_t)P.ndim * P.np * nyl * P.nsp));
    WM_TRY(rd.find("dataset", "np2", e));
    if (e.shape != std::vector<long long>{nyl, P.nsp, P.nproc}) return WM_ERR_IO;
    WM_TRY(rd.read(e, np2, sizeof(int) * (size_t)nyl * P.nsp));
    WM_TRY(rd.find("dataset", "uf", e));
    if (e.shape != std::vector<long long>{6, ghost_nx(), ghost_ny(), P.nproc}) return WM_ERR_IO;
    return rd.read(e, uf, sizeof(double) * 6 * (size_t)ghost_nx() * ghost_ny());
}

int wm_paraio_param(int n0, double wpe, double wpi, double wge, double wgi, double vti, double vte, const char *filename)
{
    if (!g_pio.init) return WM_ERR_NOT_INIT;
    if (!filename) return WM_ERR_BAD_ARG;
    const wmpio::Params &P = g_pio.P;
    const double vai = P.c * wgi / wpi, vae = P.c * wge / wpe;
    wmpio::Writer w;
    WM_TRY(w.open(P.dir, filename));
    WM_TRY(w.attr_i8("dummy_attribute", 8));
    WM_TRY(w.attr_i4("nx", P.nxge - P.nxgs + 1));
    WM_TRY(w.attr_i4("ny", P.nyge - P.nygs + 1));
    WM_TRY(w.attr_i4("np", P.np));
    WM_TRY(w.attr_f8("delx", P.delx));
    WM_TRY(w.attr_f8("delt", P.delt));
    WM_TRY(w.attr_f8("c", P.c));
    WM_TRY(w.attr_f8v("r", P.r, P.nsp));
    WM_TRY(w.attr_f8v("q", P.q, P.nsp));
    const char *names[8] = {"wpe", "wge", "wpi", "wgi", "vti", "vte", "vai", "vae"};
    const double vals[8] = {wpe, wge, wpi, wgi, vti, vte, vai, vae};
    for (int k = 0; k < 8; ++k) WM_TRY(w.attr_f8(names[k], vals[k]));
    WM_TRY(w.attr_i4("n0", n0));
    return w.close();
}

int wm_paraio_mom(double *mom, const double *uf, int it)
{
    if (!g_pio.init) return WM_ERR_NOT_INIT;
    if (!mom || !uf) return WM_ERR_BAD_ARG;
    const wmpio::Params &P = g_pio.P;
    char name[32];
    snprintf(name, sizeof name, "%07d_mom", it);
    wmpio::Writer w;
    WM_TRY(w.open(P.dir, name));
    WM_TRY(wmpio::write_head(w, P, it, {}));
    const int nx = P.nxge - P.nxgs + 1, ny = P.nyge - P.nygs + 1, nyl = rows();
    const int mx = nx + 2, my = nyl + 2, gx = ghost_nx();
    const size_t nm = (size_t)mx * my * P.nsp;
    auto M = [&](int k, int i, int j, int s) -> double & { return mom[k + 7 * (i + (size_t)mx * (j + (size_t)my * s))]; };
    std::vector<double> line;
    WM_TRY(w.dataset("den", "f8", {nx, ny, P.nsp}, "density"));
    line.resize(nx);
    for (int s = 0; s < P.nsp; ++s)
        for (int j = 1; j <= nyl; ++j) {
            for (int i = 0; i < nx; ++i) line[i] = M(0, i + 1, j, s);
            WM_TRY(w.write(line.data(), sizeof(double) * nx));
        }
    // paraio.f90:641-643 and :658-660 divide the caller's whole array, ghost cells included
    line.resize(3 * (size_t)nx);
    for (int part = 0; part < 2; ++part) {
        const int k0 = part == 0 ? 1 : 4;
        for (size_t c = 0; c < nm; ++c)
            for (int k = k0; k < k0 + 3; ++k) mom[k + 7 * c] = mom[k + 7 * c] / mom[7 * c];
        WM_TRY(w.dataset(part == 0 ? "vel" : "temp", "f8", {3, nx, ny, P.nsp}, part == 0 ? "velocity" : "temperature"));
        for (int s = 0; s < P.nsp; ++s)
            for (int j = 1; j <= nyl; ++j) {
                for (int i = 0; i < nx; ++i)
                    for (int k = 0; k < 3; ++k) line[3 * i + k] = M(k0 + k, i + 1, j, s);
                WM_TRY(w.write(line.data(), sizeof(double) * 3 * nx));
            }
    }
    WM_TRY(w.dataset("uf", "f8", {6, nx, ny}, "electromagnetic field"));
    auto U = [&](int k, int ix, int iy) { return uf[k + 6 * (ix + (size_t)gx * iy)]; };
    line.resize(6 * (size_t)nx);
    for (int j = 0; j < nyl; ++j) {
        for (int i = 0; i < nx; ++i) {
            const int ix = i + 2, iy = j + 2;
            double *t = &line[6 * i];
            t[0] = (U(0, ix, iy) + U(0, ix, iy + 1)) / 2;
            t[1] = (U(1, ix, iy) + U(1, ix + 1, iy)) / 2;
            t[2] = (U(2, ix, iy) + U(2, ix + 1, iy) + U(2, ix + 1, iy) + U(2, ix + 1, iy + 1)) / 4;
            t[3] = (U(3, ix, iy) + U(3, ix + 1, iy)) / 2;
            t[4] = (U(4, ix, iy) + U(4, ix, iy + 1)) / 2;
            t[5] = U(5, ix, iy);
        }
        WM_TRY(w.write(line.data(), sizeof(double) * line.size()));
    }
    return w.close();
}

int wm_paraio_ptcl(const double *up, const double *uf, const int *np2, int it)
{
    return write_particles_host(up, uf, np2, it, 0);
}

int wm_paraio_orb(const double *up, const double *uf, const int *np2, int it)
{
    return write_particles_host(up, uf, np2, it, 1);
}

}  // extern "C"
