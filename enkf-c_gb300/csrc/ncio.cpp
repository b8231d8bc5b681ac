// ncio.cpp -- NetCDF classic files (CDF-1, CDF-2 "64-bit offset", CDF-5
// "64-bit data") on the host, for the files around the hot path:
//   transforms.nc  (nc_createtransforms / nc_writetransforms, calc/transforms.c:54-131)
//   enkf_diag.nc   (calc/transforms.c:380-470)
//   member fields  (ncu_readfield_part, common/ncutils.c:109-530)
//   analysis files (ncu_writefield, common/ncutils.c:537-700)
// The reference does this through the NetCDF-C library; this file reads and
// writes the published classic format directly (big-endian header of
// dimensions, attributes and variables, then fixed-size variables and
// interleaved records).  No CUDA here: these entry points work without a GPU.
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/enkfg.h"

namespace {

enum {
    T_BYTE = 1, T_CHAR = 2, T_SHORT = 3, T_INT = 4, T_FLOAT = 5, T_DOUBLE = 6,
    T_UBYTE = 7, T_USHORT = 8, T_UINT = 9, T_INT64 = 10, T_UINT64 = 11
};
enum { TAG_DIM = 0x0A, TAG_VAR = 0x0B, TAG_ATT = 0x0C };

thread_local char g_err[512];

enkfg_status fail(enkfg_status st, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
enkfg_status fail(enkfg_status st, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return st;
}

int type_size(int t)
{
    switch (t) {
    case T_BYTE: case T_CHAR: case T_UBYTE: return 1;
    case T_SHORT: case T_USHORT: return 2;
    case T_INT: case T_FLOAT: case T_UINT: return 4;
    case T_DOUBLE: case T_INT64: case T_UINT64: return 8;
    default: return 0;
    }
}

long long pad4(long long n) { return (n + 3) & ~3LL; }

uint64_t get_be(const unsigned char* p, int n)
{
    uint64_t v = 0;
    for (int k = 0; k < n; ++k) v = (v << 8) | p[k];
    return v;
}

void put_be(unsigned char* p, uint64_t v, int n)
{
    for (int k = n - 1; k >= 0; --k) {
        p[k] = (unsigned char)(v & 0xff);
        v >>= 8;
    }
}

// one value of native type t (big-endian at p) as double, and as its raw
// integer image (for the bit-exact fill / missing comparisons)
double decode(const unsigned char* p, int t)
{
    uint64_t u = get_be(p, type_size(t));
    switch (t) {
    case T_BYTE: return (double)(int8_t)u;
    case T_CHAR: return (double)(uint8_t)u;
    case T_UBYTE: return (double)(uint8_t)u;
    case T_SHORT: return (double)(int16_t)u;
    case T_USHORT: return (double)(uint16_t)u;
    case T_INT: return (double)(int32_t)u;
    case T_UINT: return (double)(uint32_t)u;
    case T_INT64: return (double)(int64_t)u;
    case T_UINT64: return (double)u;
    case T_FLOAT: { uint32_t b = (uint32_t)u; float f; memcpy(&f, &b, 4); return (double)f; }
    case T_DOUBLE: { double d; memcpy(&d, &u, 8); return d; }
    default: return NAN;
    }
}

// the value as float the way NetCDF-C's get_vara_float converts it; doubles
// outside the float range become NaN (ncw_get_vara_float_fixerange,
// common/ncw.c:1078-1120)
float to_float(const unsigned char* p, int t)
{
    switch (t) {
    case T_FLOAT: { uint32_t b = (uint32_t)get_be(p, 4); float f; memcpy(&f, &b, 4); return f; }
    case T_DOUBLE: {
        uint64_t u = get_be(p, 8);
        double d;
        memcpy(&d, &u, 8);
        if (!isfinite(d) || d < -3.40282346638528859812e+38 || d > 3.40282346638528859812e+38) return NAN;
        return (float)d;
    }
    case T_INT64: return (float)(int64_t)get_be(p, 8);
    case T_UINT64: return (float)get_be(p, 8);
    case T_INT: return (float)(int32_t)get_be(p, 4);
    case T_UINT: return (float)(uint32_t)get_be(p, 4);
    default: return (float)decode(p, t);
    }
}

// n values of native type t (big-endian) as floats; the float type, the
// common case for model fields and transforms, is a byte swap
void to_float_n(const unsigned char* raw, int t, size_t n, float* out)
{
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
    if (t == T_FLOAT) {
        for (size_t q = 0; q < n; ++q) {
            uint32_t b;
            memcpy(&b, raw + q * 4, 4);
            b = __builtin_bswap32(b);
            memcpy(out + q, &b, 4);
        }
        return;
    }
#endif
    const int ts = type_size(t);
    for (size_t q = 0; q < n; ++q) out[q] = to_float(raw + q * ts, t);
}

struct Att {
    std::string name;
    int type = 0;
    long long n = 0;
    std::vector<unsigned char> raw;     // big-endian values, unpadded
    double num(long long k) const { return decode(raw.data() + k * type_size(type), type); }
};

struct Dim {
    std::string name;
    long long len = 0;                   // 0: the record dimension
};

struct Var {
    std::string name;
    std::vector<int> dimids;
    std::vector<Att> atts;
    int type = 0;
    long long vsize = 0;
    long long begin = 0;
    const Att* att(const char* nm) const
    {
        for (const Att& a : atts)
            if (a.name == nm) return &a;
        return nullptr;
    }
};

struct NcFile {
    int version = 2;
    long long numrecs = 0;
    std::vector<Dim> dims;
    std::vector<Att> gatts;
    std::vector<Var> vars;
    long long recsize = 0;

    bool is_rec(const Var& v) const { return !v.dimids.empty() && dims[v.dimids[0]].len == 0; }
    long long dimlen(const Var& v, size_t d) const
    {
        const Dim& D = dims[v.dimids[d]];
        return D.len == 0 ? numrecs : D.len;
    }
    // bytes of one record (record variables) or of the whole variable,
    // unpadded; -1 if a length is negative or the product overflows
    long long data_bytes(const Var& v) const
    {
        long long n = type_size(v.type);
        for (size_t d = is_rec(v) ? 1 : 0; d < v.dimids.size(); ++d) {
            const long long len = dims[v.dimids[d]].len;
            if (len < 0 || __builtin_mul_overflow(n, len, &n) || n > (1LL << 62)) return -1;
        }
        return n;
    }
    const Var* var(const char* nm) const
    {
        for (const Var& v : vars)
            if (v.name == nm) return &v;
        return nullptr;
    }
    // the record size; false if a variable's size is negative or overflows
    bool layout_records()
    {
        int nrec = 0;
        recsize = 0;
        for (const Var& v : vars) {
            const long long b = data_bytes(v);
            if (b < 0) return false;
            if (is_rec(v)) {
                ++nrec;
                if (__builtin_add_overflow(recsize, pad4(b), &recsize) || recsize > (1LL << 62)) return false;
            }
        }
        // a single record variable is not padded (classic format rule)
        if (nrec == 1)
            for (const Var& v : vars)
                if (is_rec(v)) recsize = data_bytes(v);
        return true;
    }
};

// ---- header parsing ------------------------------------------------------

struct Cursor {
    const unsigned char* p;
    size_t n, at = 0;
    bool ok = true;
    uint64_t take(int k)
    {
        if (at + k > n) {
            ok = false;
            return 0;
        }
        uint64_t v = get_be(p + at, k);
        at += k;
        return v;
    }
    bool bytes(long long k, std::vector<unsigned char>& out)
    {
        if (k < 0 || k > (long long)(n - at) || at + (size_t)pad4(k) > n) return ok = false;
        out.assign(p + at, p + at + k);
        at += pad4(k);
        return true;
    }
};

enkfg_status parse_header(FILE* f, const char* path, NcFile& nc)
{
    // the header is read in growing chunks until it parses
    std::vector<unsigned char> buf;
    size_t want = 1 << 16;
    for (;;) {
        buf.resize(want);
        if (fseek(f, 0, SEEK_SET) != 0) return fail(ENKFG_EINVAL, "%s: cannot seek", path);
        size_t got = fread(buf.data(), 1, want, f);
        buf.resize(got);
        Cursor c{ buf.data(), buf.size() };
        if (got < 4 || buf[0] != 'C' || buf[1] != 'D' || buf[2] != 'F')
            return fail(ENKFG_EINVAL, "%s: not a NetCDF classic file", path);
        nc = NcFile();
        nc.version = buf[3];
        if (nc.version != 1 && nc.version != 2 && nc.version != 5)
            return fail(ENKFG_EUNSUPPORTED, "%s: classic format version %d is not supported", path, nc.version);
        c.at = 4;
        const int nn = nc.version == 5 ? 8 : 4;             // NON_NEG width
        const int ob = nc.version == 1 ? 4 : 8;             // OFFSET width
        uint64_t nrec = c.take(nn);
        bool streaming = nc.version != 5 && nrec == 0xFFFFFFFFull;
        nc.numrecs = (long long)nrec;
        auto name = [&](std::string& s) {
            long long len = (long long)c.take(nn);
            std::vector<unsigned char> b;
            if (!c.ok || !c.bytes(len, b)) return false;
            s.assign(b.begin(), b.end());
            return true;
        };
        auto atts = [&](std::vector<Att>& out) {
            uint32_t tag = (uint32_t)c.take(4);
            long long na = (long long)c.take(nn);
            if (!c.ok) return false;
            if (tag == 0 && na == 0) return true;
            if (tag != TAG_ATT) return c.ok = false;
            for (long long k = 0; k < na && c.ok; ++k) {
                Att a;
                if (!name(a.name)) return false;
                a.type = (int)c.take(4);
                a.n = (long long)c.take(nn);
                if (!c.ok || type_size(a.type) == 0) return c.ok = false;
                // the count is checked against the header bytes left before
                // it is multiplied by the type size
                if (a.n < 0 || a.n > (long long)(c.n - c.at) / type_size(a.type)) return c.ok = false;
                if (!c.bytes(a.n * type_size(a.type), a.raw)) return false;
                out.push_back(std::move(a));
            }
            return c.ok;
        };
        // dimensions
        uint32_t tag = (uint32_t)c.take(4);
        long long nd = (long long)c.take(nn);
        if (c.ok && !(tag == 0 && nd == 0)) {
            if (tag != TAG_DIM) c.ok = false;
            for (long long k = 0; k < nd && c.ok; ++k) {
                Dim d;
                if (!name(d.name)) break;
                d.len = (long long)c.take(nn);
                if (d.len < 0) c.ok = false;
                nc.dims.push_back(d);
            }
        }
        if (c.ok) atts(nc.gatts);
        // variables
        if (c.ok) {
            tag = (uint32_t)c.take(4);
            long long nv = (long long)c.take(nn);
            if (c.ok && !(tag == 0 && nv == 0)) {
                if (tag != TAG_VAR) c.ok = false;
                for (long long k = 0; k < nv && c.ok; ++k) {
                    Var v;
                    if (!name(v.name)) break;
                    long long ndv = (long long)c.take(nn);
                    for (long long d = 0; d < ndv && c.ok; ++d) {
                        long long id = (long long)c.take(nn);
                        if (id < 0 || id >= (long long)nc.dims.size()) c.ok = false;
                        v.dimids.push_back((int)id);
                    }
                    if (!c.ok || !atts(v.atts)) break;
                    v.type = (int)c.take(4);
                    v.vsize = (long long)c.take(nn);
                    v.begin = (long long)c.take(ob);
                    if (type_size(v.type) == 0 || v.vsize < 0 || v.begin < 0) c.ok = false;
                    nc.vars.push_back(std::move(v));
                }
            }
        }
        if (c.ok) {
            if (!nc.layout_records())
                return fail(ENKFG_EINVAL, "%s: a variable's size in the NetCDF header overflows", path);
            for (const Var& v : nc.vars) {
                long long end;
                if (__builtin_add_overflow(v.begin, nc.data_bytes(v), &end))
                    return fail(ENKFG_EINVAL, "%s: a variable's offset in the NetCDF header overflows", path);
            }
            if (streaming) {
                // numrecs not yet written: count the complete records on disk
                long long first = -1;
                for (const Var& v : nc.vars)
                    if (nc.is_rec(v) && (first < 0 || v.begin < first)) first = v.begin;
                fseek(f, 0, SEEK_END);
                long long size = ftell(f);
                nc.numrecs = (first >= 0 && nc.recsize > 0) ? (size - first) / nc.recsize : 0;
            }
            return ENKFG_OK;
        }
        if (got < want) return fail(ENKFG_EINVAL, "%s: truncated or malformed NetCDF header", path);
        want *= 4;
        if (want > ((size_t)1 << 30)) return fail(ENKFG_EINVAL, "%s: NetCDF header too large", path);
    }
}

struct File {
    FILE* f = nullptr;
    ~File() { if (f) fclose(f); }
};

enkfg_status open_parse(const char* path, const char* mode, File& F, NcFile& nc)
{
    if (!path) return fail(ENKFG_EINVAL, "no path");
    F.f = fopen(path, mode);
    if (!F.f) return fail(ENKFG_EINVAL, "%s: %s", path, strerror(errno));
    return parse_header(F.f, path, nc);
}

// byte offset of element `idx` (all dimensions) of variable v
long long elem_offset(const NcFile& nc, const Var& v, const std::vector<long long>& idx)
{
    const bool rec = nc.is_rec(v);
    long long lin = 0;
    for (size_t d = rec ? 1 : 0; d < v.dimids.size(); ++d) lin = lin * nc.dims[v.dimids[d]].len + idx[d];
    long long off = v.begin + lin * type_size(v.type);
    if (rec) off += idx[0] * nc.recsize;
    return off;
}

// visit the contiguous runs of a hyperslab: fn(file offset, element count,
// destination element index)
template <typename F>
enkfg_status for_runs(const NcFile& nc, const Var& v, const long long* start, const long long* count, F fn)
{
    const size_t nd = v.dimids.size();
    for (size_t d = 0; d < nd; ++d)
        if (start[d] < 0 || count[d] < 0 || start[d] + count[d] > nc.dimlen(v, d))
            return fail(ENKFG_EINVAL, "%s: hyperslab [%lld, +%lld) outside dimension %zu of length %lld",
                        v.name.c_str(), start[d], count[d], d, nc.dimlen(v, d));
    long long total = 1;
    for (size_t d = 0; d < nd; ++d) total *= count[d];
    if (total == 0) return ENKFG_OK;
    // the run: the innermost dimensions covered in full, plus the next one
    size_t d0 = nd;
    long long run = 1;
    const size_t dmin = nc.is_rec(v) ? 1 : 0;   // a record breaks contiguity
    while (d0 > dmin) {
        run *= count[d0 - 1];
        --d0;
        if (count[d0] != nc.dimlen(v, d0)) break;
    }
    if (nd == 0) d0 = 0;
    std::vector<long long> idx(start, start + nd);
    for (long long done = 0; done < total; done += run) {
        enkfg_status s = fn(elem_offset(nc, v, idx), run, done);
        if (s) return s;
        // advance the outer index (dimensions before d0)
        for (long long d = (long long)d0 - 1; d >= 0; --d) {
            if (++idx[d] < start[d] + count[d]) break;
            idx[d] = start[d];
        }
    }
    return ENKFG_OK;
}

enkfg_status read_raw(FILE* f, const NcFile& nc, const Var& v, const long long* start, const long long* count,
                      std::vector<unsigned char>& out)
{
    long long total = 1;
    for (size_t d = 0; d < v.dimids.size(); ++d) total *= count[d];
    const int ts = type_size(v.type);
    out.resize((size_t)(total * ts));
    return for_runs(nc, v, start, count, [&](long long off, long long n, long long at) -> enkfg_status {
        if (fseeko(f, (off_t)off, SEEK_SET) != 0 || fread(out.data() + at * ts, ts, (size_t)n, f) != (size_t)n)
            return fail(ENKFG_EINVAL, "%s: short read at byte %lld", v.name.c_str(), off);
        return ENKFG_OK;
    });
}

// NetCDF's default fill values per type (the classic format's documented
// defaults; a classic file has no per-variable no-fill flag), as big-endian
// bytes of the type
void default_fill_raw(int t, unsigned char* out)
{
    uint64_t u = 0;
    switch (t) {
    case T_BYTE: u = 0x81; break;                                   // -127
    case T_CHAR: u = 0; break;
    case T_SHORT: u = 0x8001; break;                                // -32767
    case T_INT: u = 0x80000001u; break;                             // -2147483647
    case T_FLOAT: { const float f = 9.9692099683868690e+36f; uint32_t b; memcpy(&b, &f, 4); u = b; break; }
    case T_DOUBLE: { const double d = 9.9692099683868690e+36; memcpy(&u, &d, 8); break; }
    case T_UBYTE: u = 0xff; break;
    case T_USHORT: u = 0xffff; break;
    case T_UINT: u = 0xffffffffu; break;
    case T_INT64: u = 0x8000000000000002ull; break;                 // -9223372036854775806
    case T_UINT64: u = 0xfffffffffffffffeull; break;
    default: break;
    }
    put_be(out, u, type_size(t));
}

double default_fill(int t)
{
    switch (t) {
    case T_BYTE: return -127.0;
    case T_CHAR: return 0.0;
    case T_SHORT: return -32767.0;
    case T_INT: return -2147483647.0;
    case T_FLOAT: return (double)9.9692099683868690e+36f;
    case T_DOUBLE: return 9.9692099683868690e+36;
    case T_UBYTE: return 255.0;
    case T_USHORT: return 65535.0;
    case T_UINT: return 4294967295.0;
    case T_INT64: return -9223372036854775806.0;
    case T_UINT64: return 18446744073709551614.0;
    default: return NAN;
    }
}

// the ncu_readfield dimension rules for a structured grid (nj > 0):
// start/count of layer k of record r
enkfg_status layer_slab(const NcFile& nc, const Var& v, const char* path, int r, int k, int ni, int nj, int nk,
                        long long* start, long long* count)
{
    const int nd = (int)v.dimids.size();
    const bool rec = nc.is_rec(v);
    long long dl[4] = { 0, 0, 0, 0 };
    for (int d = 0; d < nd && d < 4; ++d) dl[d] = nc.dimlen(v, d);
    if (rec && dl[0] == 0) return fail(ENKFG_EINVAL, "%s: %s: empty record dimension", path, v.name.c_str());
    if (rec && r < 0) {
        if (dl[0] > 1) return fail(ENKFG_EINVAL, "%s: %s: not supposed to have multiple records", path, v.name.c_str());
        r = 0;
    }
    if (nd == 4) {
        if (r < 0) {
            if (dl[0] > 1) return fail(ENKFG_EINVAL, "%s: %s: not supposed to have multiple records", path, v.name.c_str());
            r = 0;
        }
        if (r >= dl[0]) return fail(ENKFG_EINVAL, "%s: %s: cannot read record %d (nr = %lld)", path, v.name.c_str(), r, dl[0]);
        if (dl[1] != nk) {
            if (dl[1] != 1)
                return fail(ENKFG_EINVAL, "%s: %s: vertical dimension %lld does not match nk = %d", path, v.name.c_str(), dl[1], nk);
            k = 0;
        }
        if (dl[3] != ni || dl[2] != nj)
            return fail(ENKFG_EINVAL, "%s: %s: horizontal dimensions %lld x %lld do not match %d x %d", path,
                        v.name.c_str(), dl[3], dl[2], ni, nj);
        const long long s[4] = { r, k, 0, 0 }, c[4] = { 1, 1, nj, ni };
        memcpy(start, s, sizeof(s));
        memcpy(count, c, sizeof(c));
    } else if (nd == 3) {
        if (dl[2] != ni || dl[1] != nj)
            return fail(ENKFG_EINVAL, "%s: %s: horizontal dimensions %lld x %lld do not match %d x %d", path,
                        v.name.c_str(), dl[2], dl[1], ni, nj);
        long long s0;
        if (!rec) {
            if (dl[0] != nk && !(dl[0] == 1 && (k <= 0 || k == nk - 1)))
                return fail(ENKFG_EINVAL, "%s: %s: vertical dimension %lld does not match nk = %d", path, v.name.c_str(), dl[0], nk);
            s0 = dl[0] == 1 ? 0 : k;
        } else {
            if (r >= dl[0]) return fail(ENKFG_EINVAL, "%s: %s: cannot read record %d (nr = %lld)", path, v.name.c_str(), r, dl[0]);
            s0 = r;                                  // a 2-D field with records: k is ignored
        }
        const long long s[3] = { s0, 0, 0 }, c[3] = { 1, nj, ni };
        memcpy(start, s, sizeof(s));
        memcpy(count, c, sizeof(c));
    } else if (nd == 2) {
        if (rec) return fail(ENKFG_EINVAL, "%s: %s: cannot read a layer from a 1-D variable", path, v.name.c_str());
        if (dl[1] != ni || dl[0] != nj)
            return fail(ENKFG_EINVAL, "%s: %s: horizontal dimensions %lld x %lld do not match %d x %d", path,
                        v.name.c_str(), dl[1], dl[0], ni, nj);
        const long long s[2] = { 0, 0 }, c[2] = { nj, ni };
        memcpy(start, s, sizeof(s));
        memcpy(count, c, sizeof(c));
    } else {
        return fail(ENKFG_EINVAL, "%s: %s: cannot read a 2-D field from %d dimensions", path, v.name.c_str(), nd);
    }
    return ENKFG_OK;
}

// ---- writing -------------------------------------------------------------

struct Writer {
    std::vector<unsigned char> h;
    int version;
    int nn() const { return version == 5 ? 8 : 4; }
    void u(uint64_t v, int k)
    {
        size_t at = h.size();
        h.resize(at + k);
        put_be(h.data() + at, v, k);
    }
    void bytes(const void* p, size_t n)
    {
        const unsigned char* b = (const unsigned char*)p;
        h.insert(h.end(), b, b + n);
        while (h.size() % 4) h.push_back(0);
    }
    void name(const std::string& s)
    {
        u(s.size(), nn());
        bytes(s.data(), s.size());
    }
    void atts(const std::vector<Att>& a)
    {
        if (a.empty()) {
            u(0, 4);
            u(0, nn());
            return;
        }
        u(TAG_ATT, 4);
        u(a.size(), nn());
        for (const Att& x : a) {
            name(x.name);
            u(x.type, 4);
            u(x.n, nn());
            bytes(x.raw.data(), x.raw.size());
        }
    }
    void header(const NcFile& nc)
    {
        h.clear();
        const char magic[4] = { 'C', 'D', 'F', (char)nc.version };
        h.insert(h.end(), magic, magic + 4);
        u(nc.numrecs, nn());
        if (nc.dims.empty()) {
            u(0, 4);
            u(0, nn());
        } else {
            u(TAG_DIM, 4);
            u(nc.dims.size(), nn());
            for (const Dim& d : nc.dims) {
                name(d.name);
                u(d.len, nn());
            }
        }
        atts(nc.gatts);
        if (nc.vars.empty()) {
            u(0, 4);
            u(0, nn());
        } else {
            u(TAG_VAR, 4);
            u(nc.vars.size(), nn());
            for (const Var& v : nc.vars) {
                name(v.name);
                u(v.dimids.size(), nn());
                for (int id : v.dimids) u(id, nn());
                atts(v.atts);
                u(v.type, 4);
                u(v.vsize, nn());
                u(v.begin, version == 1 ? 4 : 8);
            }
        }
    }
};

Att text_att(const char* nm, const char* s)
{
    Att a;
    a.name = nm;
    a.type = T_CHAR;
    a.n = (long long)strlen(s);
    a.raw.assign(s, s + a.n);
    return a;
}

Att int_att(const char* nm, int v)
{
    Att a;
    a.name = nm;
    a.type = T_INT;
    a.n = 1;
    a.raw.resize(4);
    put_be(a.raw.data(), (uint32_t)v, 4);
    return a;
}

// a file of fixed-size variables only: header, then the variables' data in
// definition order, each padded to 4 bytes
struct FixedVar {
    const void* data;           // host values (int32 or float), native order
};

enkfg_status write_fixed(const char* path, NcFile& nc, const std::vector<FixedVar>& data)
{
    // 64-bit offset format unless a variable needs the 64-bit data format
    nc.version = 2;
    for (const Var& v : nc.vars)
        if (nc.data_bytes(v) > 0xFFFFFFFFLL - 4) nc.version = 5;
    for (Var& v : nc.vars) v.vsize = pad4(nc.data_bytes(v));
    Writer w{ {}, nc.version };
    w.header(nc);                                    // sizes the header
    long long off = (long long)w.h.size();
    for (Var& v : nc.vars) {
        v.begin = off;
        off += v.vsize;
    }
    w.header(nc);
    FILE* f = fopen(path, "wb");
    if (!f) return fail(ENKFG_EINVAL, "%s: %s", path, strerror(errno));
    File F;
    F.f = f;
    if (fwrite(w.h.data(), 1, w.h.size(), f) != w.h.size()) return fail(ENKFG_EINVAL, "%s: write failed", path);
    std::vector<unsigned char> buf;
    for (size_t k = 0; k < nc.vars.size(); ++k) {
        const Var& v = nc.vars[k];
        const long long n = nc.data_bytes(v) / 4;    // int32 and float only here
        const uint32_t* src = (const uint32_t*)data[k].data;
        if (!src) {
            // no data yet: the variable's space is reserved (written row by
            // row later); the file is extended to its full size at the end
            if (fseeko(f, (off_t)v.vsize, SEEK_CUR) != 0) return fail(ENKFG_EINVAL, "%s: seek failed", path);
            continue;
        }
        const long long chunk = 1 << 20;
        for (long long a = 0; a < n; a += chunk) {
            const long long m = n - a < chunk ? n - a : chunk;
            buf.resize((size_t)m * 4);
            for (long long q = 0; q < m; ++q) put_be(buf.data() + q * 4, src[a + q], 4);
            if (fwrite(buf.data(), 4, (size_t)m, f) != (size_t)m) return fail(ENKFG_EINVAL, "%s: write failed", path);
        }
        const long long padn = v.vsize - n * 4;
        const unsigned char z[4] = { 0, 0, 0, 0 };
        if (padn > 0 && fwrite(z, 1, (size_t)padn, f) != (size_t)padn) return fail(ENKFG_EINVAL, "%s: write failed", path);
    }
    const long long end = ftello(f);
    if (end != off) {
        const unsigned char z = 0;
        if (fseeko(f, (off_t)(off - 1), SEEK_SET) != 0 || fwrite(&z, 1, 1, f) != 1)
            return fail(ENKFG_EINVAL, "%s: write failed", path);
    }
    if (fflush(f) != 0) return fail(ENKFG_EINVAL, "%s: write failed", path);
    return ENKFG_OK;
}

// big-endian images of host values written into a hyperslab of a float or
// int variable of an open file
enkfg_status write_slab(FILE* f, const NcFile& nc, const Var& v, const long long* start, const long long* count,
                        const void* host)
{
    long long total = 1;
    for (size_t d = 0; d < v.dimids.size(); ++d) total *= count[d];
    std::vector<unsigned char> raw((size_t)total * 4);
    const uint32_t* src = (const uint32_t*)host;
    for (long long q = 0; q < total; ++q) put_be(raw.data() + q * 4, src[q], 4);
    return for_runs(nc, v, start, count, [&](long long off, long long m, long long at) -> enkfg_status {
        if (fseeko(f, (off_t)off, SEEK_SET) != 0 || fwrite(raw.data() + at * 4, 4, (size_t)m, f) != (size_t)m)
            return fail(ENKFG_EINVAL, "%s: write failed at byte %lld", v.name.c_str(), off);
        return ENKFG_OK;
    });
}

Var fixed_var(const char* nm, int type, std::initializer_list<int> dimids)
{
    Var v;
    v.name = nm;
    v.type = type;
    v.dimids.assign(dimids.begin(), dimids.end());
    return v;
}

// A float stored into an integer variable as NetCDF's put conversion does
// it: a C conversion (truncation toward zero), with values outside the type's
// range refused (NC_ERANGE, on which the reference's writer stops).
bool pack_integer(float x, int t, uint64_t& out)
{
    if (x != x) return false;
    switch (t) {
    case T_BYTE:
        if (x < -128.0f || x > 127.0f) return false;
        out = (uint8_t)(int8_t)x;
        return true;
    case T_UBYTE:
        if (x < 0.0f || x > 255.0f) return false;
        out = (uint8_t)x;
        return true;
    case T_SHORT:
        if (x < -32768.0f || x > 32767.0f) return false;
        out = (uint16_t)(int16_t)x;
        return true;
    case T_USHORT:
        if (x < 0.0f || x > 65535.0f) return false;
        out = (uint16_t)x;
        return true;
    case T_INT:
        if (x < -2147483648.0f || x >= 2147483648.0f) return false;
        out = (uint32_t)(int32_t)x;
        return true;
    case T_UINT:
        if (x < 0.0f || x >= 4294967296.0f) return false;
        out = (uint32_t)x;
        return true;
    case T_INT64:
        if (x < -9223372036854775808.0f || x >= 9223372036854775808.0f) return false;
        out = (uint64_t)(int64_t)x;
        return true;
    case T_UINT64:
        if (x < 0.0f || x >= 18446744073709551616.0f) return false;
        out = (uint64_t)x;
        return true;
    default:
        return false;
    }
}

// The value rules of ncu_readfield / ncu_read3dfield (common/ncutils.c:
// 300-530, 1015-1245): values equal to the fill value (the attribute, else
// the type's default) or to missing_value, and values outside valid_min /
// valid_max / valid_range, become NaN, compared on the native values
// (integers and bit patterns alike); then scale_factor and add_offset as
// floats.  ncu_read3dfield masks only when one of those five attributes is
// present (only_with_atts).
void apply_read_rules(const Var& V, const std::vector<unsigned char>& raw, float* v, bool only_with_atts)
{
    const int t = V.type, ts = type_size(t);
    const size_t n = raw.size() / ts;
    auto same = [&](const unsigned char* p, const Att& a) {
        if (a.n != 1) return false;
        if (a.type == t) return memcmp(p, a.raw.data(), ts) == 0;
        return decode(p, t) == a.num(0);
    };
    const Att* fillv = V.att("_FillValue");
    unsigned char dfill[8];
    default_fill_raw(t, dfill);
    const Att* miss = V.att("missing_value");
    const Att* vmin = V.att("valid_min");
    const Att* vmax = V.att("valid_max");
    const Att* vrng = V.att("valid_range");
    const bool mask = !only_with_atts || fillv || miss || vmin || vmax || vrng;
    if (vrng && vrng->n != 2) vrng = nullptr;
    for (size_t q = 0; mask && q < n; ++q) {
        const unsigned char* p = raw.data() + q * ts;
        bool out = fillv ? same(p, *fillv) : memcmp(p, dfill, ts) == 0;
        if (!out && miss) out = same(p, *miss);
        if (!out && (vmin || vmax || vrng)) {
            const double x = decode(p, t);
            if (vmin && vmin->n == 1 && x < vmin->num(0)) out = true;
            if (vmax && vmax->n == 1 && x > vmax->num(0)) out = true;
            if (vrng && (x < vrng->num(0) || x > vrng->num(1))) out = true;
        }
        if (out) v[q] = NAN;
    }
    if (const Att* a = V.att("scale_factor")) {
        const float sf = (float)a->num(0);
        for (size_t q = 0; q < n; ++q) v[q] *= sf;
    }
    if (const Att* a = V.att("add_offset")) {
        const float ao = (float)a->num(0);
        for (size_t q = 0; q < n; ++q) v[q] += ao;
    }
}

// the entry points: no C++ exception crosses the C ABI
template <typename F>
enkfg_status guarded(F f)
{
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(ENKFG_ENOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(ENKFG_EINVAL, "%s", e.what());
    }
}

}  // namespace

extern "C" {

ENKFG_API const char* enkfg_nc_last_error(void)
{
    return g_err;
}

// the transforms.nc layout of nc_createtransforms (calc/transforms.c:54-94)
static NcFile transforms_file(int nj, int ni, int nmem_dynamic, int nmem, bool with_T, int stride,
                              const char* grid_name)
{
    NcFile nc;
    nc.dims.push_back({ "j", nj });
    nc.dims.push_back({ "i", ni });
    if (with_T) {
        nc.dims.push_back({ "m_dyn", nmem_dynamic });
        nc.dims.push_back({ "m", nmem });
        nc.vars.push_back(fixed_var("T", T_FLOAT, { 0, 1, 2, 3 }));
        nc.vars.push_back(fixed_var("w", T_FLOAT, { 0, 1, 3 }));
    } else {
        nc.dims.push_back({ "m", nmem });
        nc.vars.push_back(fixed_var("w", T_FLOAT, { 0, 1, 2 }));
    }
    nc.gatts.push_back(int_att("stride", stride));
    nc.gatts.push_back(text_att("grid_name", grid_name ? grid_name : ""));
    return nc;
}

static enkfg_status impl_write_transforms(const char* path, int nj, int ni, int nmem_dynamic, int nmem,
                                          const float* T, const float* w, int stride, const char* grid_name)
{
    if (nj < 1 || ni < 1 || nmem < 1 || !w || (T && (nmem_dynamic < 1 || nmem_dynamic > nmem)))
        return fail(ENKFG_EINVAL, "bad transforms dimensions %d x %d, m_dyn %d, m %d", nj, ni, nmem_dynamic, nmem);
    NcFile nc = transforms_file(nj, ni, nmem_dynamic, nmem, T != nullptr, stride, grid_name);
    std::vector<FixedVar> data;
    data.reserve(2);
    if (T) data.push_back(FixedVar{ T });
    data.push_back(FixedVar{ w });
    return write_fixed(path, nc, data);
}

static enkfg_status impl_create_transforms(const char* path, int nj, int ni, int nmem_dynamic, int nmem, int with_T,
                                           int stride, const char* grid_name)
{
    if (nj < 1 || ni < 1 || nmem < 1 || (with_T && (nmem_dynamic < 1 || nmem_dynamic > nmem)))
        return fail(ENKFG_EINVAL, "bad transforms dimensions %d x %d, m_dyn %d, m %d", nj, ni, nmem_dynamic, nmem);
    NcFile nc = transforms_file(nj, ni, nmem_dynamic, nmem, with_T != 0, stride, grid_name);
    std::vector<FixedVar> data(nc.vars.size(), FixedVar{ nullptr });
    return write_fixed(path, nc, data);
}

static enkfg_status impl_write_transforms_row(const char* path, int j, const float* Tj, const float* wj)
{
    File F;
    NcFile nc;
    enkfg_status s = open_parse(path, "r+b", F, nc);
    if (s) return s;
    const Var* W = nc.var("w");
    const Var* T = nc.var("T");
    if (!W || W->type != T_FLOAT || W->dimids.size() != 3 || nc.is_rec(*W))
        return fail(ENKFG_EINVAL, "%s: not a transforms file (no float w [j][i][m])", path);
    const long long nj = nc.dimlen(*W, 0), ni = nc.dimlen(*W, 1), m = nc.dimlen(*W, 2);
    if (j < 0 || j >= nj) return fail(ENKFG_EINVAL, "%s: row %d outside 0..%lld", path, j, nj - 1);
    if (!wj || (T && !Tj)) return fail(ENKFG_EINVAL, "%s: row data missing", path);
    if (T) {
        if (T->type != T_FLOAT || T->dimids.size() != 4 || nc.dimlen(*T, 0) != nj || nc.dimlen(*T, 1) != ni ||
            nc.dimlen(*T, 3) != m)
            return fail(ENKFG_EINVAL, "%s: T does not match w", path);
        const long long st4[4] = { j, 0, 0, 0 }, ct4[4] = { 1, ni, nc.dimlen(*T, 2), m };
        if ((s = write_slab(F.f, nc, *T, st4, ct4, Tj))) return s;
    }
    const long long st3[3] = { j, 0, 0 }, ct3[3] = { 1, ni, m };
    return write_slab(F.f, nc, *W, st3, ct3, wj);
}

static enkfg_status impl_write_diag(const char* path, int nj, int ni, int ntypes, const char* const* type_names,
                                           int stride, const int* nlobs, const float* dfs, const float* srf,
                                           const int* pnlobs, const float* pdfs, const float* psrf)
{
    if (nj < 1 || ni < 1 || ntypes < 1 || !type_names || !nlobs || !dfs || !srf || !pnlobs || !pdfs || !psrf)
        return fail(ENKFG_EINVAL, "bad diagnostics arguments");
    NcFile nc;
    nc.dims.push_back({ "nobstypes", ntypes });
    nc.dims.push_back({ "j", nj });
    nc.dims.push_back({ "i", ni });
    Var v;
    v = fixed_var("nlobs", T_INT, { 1, 2 });
    v.atts.push_back(text_att("long_name", "number of local observations"));
    nc.vars.push_back(v);
    v = fixed_var("dfs", T_FLOAT, { 1, 2 });
    v.atts.push_back(text_att("long_name", "local DFS (Degrees of Freedom for Signal)"));
    v.atts.push_back(text_att("comment", "DFS = trace(KH) for vanilla KF"));
    nc.vars.push_back(v);
    v = fixed_var("srf", T_FLOAT, { 1, 2 });
    v.atts.push_back(text_att("long_name", "local SRF (Spread Reduction Factor)"));
    v.atts.push_back(text_att("comment", "SRF = (forecast spread / analysis spread) - 1 for vanilla ETKF"));
    nc.vars.push_back(v);
    v = fixed_var("pnlobs", T_INT, { 0, 1, 2 });
    v.atts.push_back(text_att("long_name", "partial number of local observations"));
    nc.vars.push_back(v);
    v = fixed_var("pdfs", T_FLOAT, { 0, 1, 2 });
    v.atts.push_back(text_att("long_name", "partial local DFS"));
    nc.vars.push_back(v);
    v = fixed_var("psrf", T_FLOAT, { 0, 1, 2 });
    v.atts.push_back(text_att("long_name", "partial local SRF"));
    nc.vars.push_back(v);
    nc.gatts.push_back(int_att("stride", stride));
    for (int t = 0; t < ntypes; ++t) {
        if (!type_names[t] || !type_names[t][0]) return fail(ENKFG_EINVAL, "observation type %d has no name", t);
        nc.gatts.push_back(int_att(type_names[t], t));
    }
    return write_fixed(path, nc, { { nlobs }, { dfs }, { srf }, { pnlobs }, { pdfs }, { psrf } });
}

static enkfg_status impl_inq_var(const char* path, const char* var, int* ndims, long long* dims, int* type,
                                        int* has_record)
{
    File F;
    NcFile nc;
    enkfg_status s = open_parse(path, "rb", F, nc);
    if (s) return s;
    const Var* v = var ? nc.var(var) : nullptr;
    if (!v) return fail(ENKFG_EINVAL, "%s: no variable \"%s\"", path, var ? var : "(null)");
    if ((int)v->dimids.size() > ENKFG_NC_MAXDIMS)
        return fail(ENKFG_EUNSUPPORTED, "%s: %s has more than %d dimensions", path, var, ENKFG_NC_MAXDIMS);
    if (ndims) *ndims = (int)v->dimids.size();
    if (dims)
        for (size_t d = 0; d < v->dimids.size(); ++d) dims[d] = nc.dimlen(*v, d);
    if (type) *type = v->type;
    if (has_record) *has_record = nc.is_rec(*v) ? 1 : 0;
    return ENKFG_OK;
}

static enkfg_status impl_get_vara_float(const char* path, const char* var, const long long* start,
                                               const long long* count, float* out)
{
    File F;
    NcFile nc;
    enkfg_status s = open_parse(path, "rb", F, nc);
    if (s) return s;
    const Var* v = var ? nc.var(var) : nullptr;
    if (!v) return fail(ENKFG_EINVAL, "%s: no variable \"%s\"", path, var ? var : "(null)");
    if (v->type == T_CHAR) return fail(ENKFG_EINVAL, "%s: %s is text", path, var);
    if (!v->dimids.empty() && (!start || !count)) return fail(ENKFG_EINVAL, "start and count are required");
    std::vector<unsigned char> raw;
    if ((s = read_raw(F.f, nc, *v, start, count, raw))) return s;
    const int ts = type_size(v->type);
    const size_t n = raw.size() / ts;
    to_float_n(raw.data(), v->type, n, out);
    return ENKFG_OK;
}

static enkfg_status impl_read_layer(const char* path, const char* var, int r, int k, int ni, int nj, int nk,
                                           float* v)
{
    if (ni < 1 || nj < 1 || nk < 1 || !v) return fail(ENKFG_EINVAL, "bad layer arguments");
    File F;
    NcFile nc;
    enkfg_status s = open_parse(path, "rb", F, nc);
    if (s) return s;
    const Var* V = var ? nc.var(var) : nullptr;
    if (!V) return fail(ENKFG_EINVAL, "%s: no variable \"%s\"", path, var ? var : "(null)");
    if (V->type == T_CHAR) return fail(ENKFG_EINVAL, "%s: %s is text", path, var);
    long long start[4], count[4];
    if ((s = layer_slab(nc, *V, path, r, k, ni, nj, nk, start, count))) return s;
    std::vector<unsigned char> raw;
    if ((s = read_raw(F.f, nc, *V, start, count, raw))) return s;
    const int t = V->type, ts = type_size(t);
    const size_t n = raw.size() / ts;
    to_float_n(raw.data(), t, n, v);

    apply_read_rules(*V, raw, v, false);
    return ENKFG_OK;
}

static enkfg_status impl_read_field3d(const char* path, const char* var, int r, int ni, int nj, int nk, float* v)
{
    if (ni < 1 || nj < 1 || nk < 1 || !v) return fail(ENKFG_EINVAL, "bad field arguments");
    File F;
    NcFile nc;
    enkfg_status s = open_parse(path, "rb", F, nc);
    if (s) return s;
    const Var* V = var ? nc.var(var) : nullptr;
    if (!V) return fail(ENKFG_EINVAL, "%s: no variable \"%s\"", path, var ? var : "(null)");
    if (V->type == T_CHAR) return fail(ENKFG_EINVAL, "%s: %s is text", path, var);
    // the ncu_read3dfield dimension rules on a structured grid
    // (common/ncutils.c:923-990): [r][k][j][i] or [k][j][i]
    const int nd = (int)V->dimids.size();
    const bool rec = nc.is_rec(*V);
    long long dl[4] = { 0, 0, 0, 0 };
    for (int d = 0; d < nd && d < 4; ++d) dl[d] = nc.dimlen(*V, d);
    if (rec && dl[0] == 0) return fail(ENKFG_EINVAL, "%s: %s: empty record dimension", path, var);
    long long start[4] = { 0, 0, 0, 0 }, count[4] = { 0, 0, 0, 0 };
    if (nd == 4) {
        if (r < 0) {
            if (dl[0] > 1) return fail(ENKFG_EINVAL, "%s: %s: not supposed to have multiple records", path, var);
            r = 0;
        }
        if (r >= dl[0]) return fail(ENKFG_EINVAL, "%s: %s: cannot read record %d (nr = %lld)", path, var, r, dl[0]);
        if (dl[3] != ni || dl[2] != nj || dl[1] != nk)
            return fail(ENKFG_EINVAL, "%s: %s: dimensions %lld x %lld x %lld do not match %d x %d x %d", path, var,
                        dl[3], dl[2], dl[1], ni, nj, nk);
        const long long s4[4] = { r, 0, 0, 0 }, c4[4] = { 1, nk, nj, ni };
        memcpy(start, s4, sizeof(s4));
        memcpy(count, c4, sizeof(c4));
    } else if (nd == 3) {
        if (rec) return fail(ENKFG_EINVAL, "%s: %s: a 2-D variable with records is not a 3-D field", path, var);
        if (r > 0) return fail(ENKFG_EINVAL, "%s: %s: no record %d in a 3-dimensional variable", path, var, r);
        if (dl[2] != ni || dl[1] != nj || dl[0] != nk)
            return fail(ENKFG_EINVAL, "%s: %s: dimensions %lld x %lld x %lld do not match %d x %d x %d", path, var,
                        dl[2], dl[1], dl[0], ni, nj, nk);
        const long long s3[3] = { 0, 0, 0 }, c3[3] = { nk, nj, ni };
        memcpy(start, s3, sizeof(s3));
        memcpy(count, c3, sizeof(c3));
    } else {
        return fail(ENKFG_EINVAL, "%s: %s: cannot read a 3-D field from %d dimensions", path, var, nd);
    }
    std::vector<unsigned char> raw;
    if ((s = read_raw(F.f, nc, *V, start, count, raw))) return s;
    const int t = V->type, ts = type_size(t);
    const size_t n = raw.size() / ts;
    for (size_t q = 0; q < n; ++q) {
        v[q] = to_float(raw.data() + q * ts, t);
        // a double beyond the float range stops the reference's read
        // (ncw_get_vara_float without the range fix)
        if (t == T_DOUBLE && v[q] != v[q] && decode(raw.data() + q * ts, t) == decode(raw.data() + q * ts, t))
            return fail(ENKFG_EINVAL, "%s: %s: value %zu outside the float range", path, var, q);
    }
    apply_read_rules(*V, raw, v, true);
    return ENKFG_OK;
}

static enkfg_status impl_write_layer(const char* path, const char* var, int k, int ni, int nj, int nk,
                                            const float* v)
{
    if (ni < 1 || nj < 1 || nk < 1 || !v) return fail(ENKFG_EINVAL, "bad layer arguments");
    File F;
    NcFile nc;
    enkfg_status s = open_parse(path, "r+b", F, nc);
    if (s) return s;
    const Var* V = var ? nc.var(var) : nullptr;
    if (!V) return fail(ENKFG_EINVAL, "%s: no variable \"%s\"", path, var ? var : "(null)");
    if (V->type == T_CHAR) return fail(ENKFG_EUNSUPPORTED, "%s: %s: a text variable", path, var);
    // the ncu_writefield dimension rules (common/ncutils.c:553-640): the last
    // record of a record variable, layer k otherwise
    const int nd = (int)V->dimids.size();
    const bool rec = nc.is_rec(*V);
    long long dl[4] = { 0, 0, 0, 0 };
    for (int d = 0; d < nd && d < 4; ++d) dl[d] = nc.dimlen(*V, d);
    long long start[4] = { 0, 0, 0, 0 }, count[4] = { 0, 0, 0, 0 };
    if (nd == 4) {
        if (!rec && dl[0] != 1)
            return fail(ENKFG_EINVAL, "%s: %s: the first of 4 dimensions must be unlimited or of length 1", path, var);
        if (dl[1] != nk) return fail(ENKFG_EINVAL, "%s: %s: vertical dimension %lld does not match nk = %d", path, var, dl[1], nk);
        if (dl[3] != ni || dl[2] != nj) return fail(ENKFG_EINVAL, "%s: %s: horizontal dimensions do not match", path, var);
        if (dl[0] == 0) return fail(ENKFG_EUNSUPPORTED, "%s: %s: no record to write into", path, var);
        const long long s4[4] = { dl[0] - 1, k, 0, 0 }, c4[4] = { 1, 1, nj, ni };
        memcpy(start, s4, sizeof(s4));
        memcpy(count, c4, sizeof(c4));
    } else if (nd == 3) {
        if (dl[2] != ni || dl[1] != nj) return fail(ENKFG_EINVAL, "%s: %s: horizontal dimensions do not match", path, var);
        long long s0;
        if (!rec) {
            if (dl[0] != nk && !(dl[0] == 1 && (k == 0 || k == nk - 1)))
                return fail(ENKFG_EINVAL, "%s: %s: vertical dimension %lld does not match nk = %d", path, var, dl[0], nk);
            s0 = k;
            if (dl[0] == 1) s0 = 0;
        } else {
            if (dl[0] == 0) return fail(ENKFG_EUNSUPPORTED, "%s: %s: no record to write into", path, var);
            s0 = dl[0] - 1;
        }
        const long long s3[3] = { s0, 0, 0 }, c3[3] = { 1, nj, ni };
        memcpy(start, s3, sizeof(s3));
        memcpy(count, c3, sizeof(c3));
    } else if (nd == 2) {
        if (rec) return fail(ENKFG_EINVAL, "%s: %s: cannot write a layer to a 1-D variable", path, var);
        if (dl[1] != ni || dl[0] != nj) return fail(ENKFG_EINVAL, "%s: %s: horizontal dimensions do not match", path, var);
        const long long s2[2] = { 0, 0 }, c2[2] = { nj, ni };
        memcpy(start, s2, sizeof(s2));
        memcpy(count, c2, sizeof(c2));
    } else {
        return fail(ENKFG_EINVAL, "%s: %s: cannot write a 2-D field to %d dimensions", path, var, nd);
    }
    // unpacking in reverse, clamping to the valid range, NaN to the fill
    // value (then missing_value), as floats (ncutils.c:655-700)
    const size_t n = (size_t)ni * nj;
    std::vector<float> x(v, v + n);
    if (const Att* a = V->att("add_offset")) {
        const float ao = (float)a->num(0);
        for (float& q : x) q -= ao;
    }
    if (const Att* a = V->att("scale_factor")) {
        const float sf = (float)a->num(0);
        for (float& q : x) q /= sf;
    }
    if (const Att* a = V->att("valid_min"))
        if (a->n == 1)
            for (float& q : x) if (q < (float)a->num(0)) q = (float)a->num(0);
    if (const Att* a = V->att("valid_max"))
        if (a->n == 1)
            for (float& q : x) if (q > (float)a->num(0)) q = (float)a->num(0);
    if (const Att* a = V->att("valid_range"))
        if (a->n == 2)
            for (float& q : x) {
                if (q < (float)a->num(0)) q = (float)a->num(0);
                else if (q > (float)a->num(1)) q = (float)a->num(1);
            }
    const Att* fa = V->att("_FillValue");
    const float fill = fa && fa->n == 1 ? (float)fa->num(0) : (float)default_fill(V->type);
    for (float& q : x)
        if (isnan(q)) q = fill;
    if (const Att* a = V->att("missing_value"))
        if (a->n == 1)
            for (float& q : x) if (isnan(q)) q = (float)a->num(0);
    const int ts = type_size(V->type);
    std::vector<unsigned char> raw(n * ts);
    for (size_t q = 0; q < n; ++q) {
        if (V->type == T_FLOAT) {
            uint32_t b;
            memcpy(&b, &x[q], 4);
            put_be(raw.data() + q * 4, b, 4);
        } else if (V->type == T_DOUBLE) {
            const double d = (double)x[q];
            uint64_t b;
            memcpy(&b, &d, 8);
            put_be(raw.data() + q * 8, b, 8);
        } else {
            uint64_t b;
            if (!pack_integer(x[q], V->type, b))
                return fail(ENKFG_EINVAL, "%s: %s: value %g at %zu outside the range of the variable's type", path,
                            var, (double)x[q], q);
            put_be(raw.data() + q * ts, b, ts);
        }
    }
    return for_runs(nc, *V, start, count, [&](long long off, long long m, long long at) -> enkfg_status {
        if (fseeko(F.f, (off_t)off, SEEK_SET) != 0 || fwrite(raw.data() + at * ts, ts, (size_t)m, F.f) != (size_t)m)
            return fail(ENKFG_EINVAL, "%s: write failed at byte %lld", path, off);
        return ENKFG_OK;
    });
}



ENKFG_API enkfg_status enkfg_nc_write_transforms(const char* path, int nj, int ni, int nmem_dynamic, int nmem, const float* T, const float* w, int stride, const char* grid_name)
{
    return guarded([&] { return impl_write_transforms(path, nj, ni, nmem_dynamic, nmem, T, w, stride, grid_name); });
}

ENKFG_API enkfg_status enkfg_nc_create_transforms(const char* path, int nj, int ni, int nmem_dynamic, int nmem,
                                                  int with_T, int stride, const char* grid_name)
{
    return guarded([&] { return impl_create_transforms(path, nj, ni, nmem_dynamic, nmem, with_T, stride, grid_name); });
}

ENKFG_API enkfg_status enkfg_nc_write_transforms_row(const char* path, int j, const float* Tj, const float* wj)
{
    return guarded([&] { return impl_write_transforms_row(path, j, Tj, wj); });
}

ENKFG_API enkfg_status enkfg_nc_write_diag(const char* path, int nj, int ni, int ntypes, const char* const* type_names, int stride, const int* nlobs, const float* dfs, const float* srf, const int* pnlobs, const float* pdfs, const float* psrf)
{
    return guarded([&] { return impl_write_diag(path, nj, ni, ntypes, type_names, stride, nlobs, dfs, srf, pnlobs, pdfs, psrf); });
}

ENKFG_API enkfg_status enkfg_nc_inq_var(const char* path, const char* var, int* ndims, long long* dims, int* type, int* has_record)
{
    return guarded([&] { return impl_inq_var(path, var, ndims, dims, type, has_record); });
}

ENKFG_API enkfg_status enkfg_nc_get_vara_float(const char* path, const char* var, const long long* start, const long long* count, float* out)
{
    return guarded([&] { return impl_get_vara_float(path, var, start, count, out); });
}

ENKFG_API enkfg_status enkfg_nc_read_layer(const char* path, const char* var, int r, int k, int ni, int nj, int nk, float* v)
{
    return guarded([&] { return impl_read_layer(path, var, r, k, ni, nj, nk, v); });
}

ENKFG_API enkfg_status enkfg_nc_read_field3d(const char* path, const char* var, int r, int ni, int nj, int nk, float* v)
{
    return guarded([&] { return impl_read_field3d(path, var, r, ni, nj, nk, v); });
}

ENKFG_API enkfg_status enkfg_nc_write_layer(const char* path, const char* var, int k, int ni, int nj, int nk, const float* v)
{
    return guarded([&] { return impl_write_layer(path, var, k, ni, nj, nk, v); });
}
}  // extern "C"
