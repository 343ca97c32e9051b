// wf_netcdf.cpp -- reader and writer of the netCDF classic binary formats (CDF-1, CDF-2, CDF-5)
// for Wflow's static maps, forcing and state files (include/wflow_gb300_nc.h).
//
// Layout (netCDF classic format specification): magic "CDF" + version byte, the number of
// records, then three tagged lists -- dimensions (tag 10), global attributes (tag 12),
// variables (tag 11, each with its own attribute list, type, size and data offset). Integers
// are big-endian; counts, lengths, dimension ids and sizes are 4 bytes in CDF-1/2 and 8 bytes in
// CDF-5; data offsets are 4 bytes in CDF-1 and 8 in CDF-2/5. Names and attribute values are
// padded to 4 bytes. Fixed-size variables are stored contiguously in definition order; the
// record variables follow, interleaved: record r of variable v starts at begin(v) + r * recsize,
// where recsize is the sum of the record variables' padded sizes (a single record variable is
// not padded).
#include "wflow_gb300_nc.h"

#include <sys/types.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "wflow_gb300.h"

namespace {

thread_local std::string g_nc_error;

constexpr int32_t TAG_DIMENSION = 10;
constexpr int32_t TAG_VARIABLE = 11;
constexpr int32_t TAG_ATTRIBUTE = 12;
constexpr int kMaxDims = 16;

int type_size(int32_t t) {
    switch (t) {
        case WF_NC_BYTE: case WF_NC_CHAR: case WF_NC_UBYTE: return 1;
        case WF_NC_SHORT: case WF_NC_USHORT: return 2;
        case WF_NC_INT: case WF_NC_FLOAT: case WF_NC_UINT: return 4;
        case WF_NC_DOUBLE: case WF_NC_INT64: case WF_NC_UINT64: return 8;
        default: return 0;
    }
}

// default fill values of the netCDF specification
double default_fill(int32_t t) {
    switch (t) {
        case WF_NC_BYTE: return -127.0;
        case WF_NC_CHAR: return 0.0;
        case WF_NC_SHORT: return -32767.0;
        case WF_NC_INT: return -2147483647.0;
        case WF_NC_FLOAT: return (double)9.9692099683868690e+36f;
        case WF_NC_DOUBLE: return 9.9692099683868690e+36;
        case WF_NC_UBYTE: return 255.0;
        case WF_NC_USHORT: return 65535.0;
        case WF_NC_UINT: return 4294967295.0;
        case WF_NC_INT64: return -9223372036854775806.0;
        case WF_NC_UINT64: return 18446744073709551614.0;
        default: return 0.0;
    }
}

int64_t pad4(int64_t n) { return (n + 3) / 4 * 4; }

// big-endian encode / decode of one value of type t
void put_be(uint8_t* p, uint64_t v, int n) {
    for (int i = n - 1; i >= 0; --i) {
        p[i] = (uint8_t)(v & 0xff);
        v >>= 8;
    }
}
uint64_t get_be(const uint8_t* p, int n) {
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v = (v << 8) | p[i];
    return v;
}

double decode_value(const uint8_t* p, int32_t t) {
    switch (t) {
        case WF_NC_BYTE: return (double)(int8_t)p[0];
        case WF_NC_CHAR: return (double)p[0];
        case WF_NC_UBYTE: return (double)p[0];
        case WF_NC_SHORT: return (double)(int16_t)(uint16_t)get_be(p, 2);
        case WF_NC_USHORT: return (double)(uint16_t)get_be(p, 2);
        case WF_NC_INT: return (double)(int32_t)(uint32_t)get_be(p, 4);
        case WF_NC_UINT: return (double)(uint32_t)get_be(p, 4);
        case WF_NC_INT64: return (double)(int64_t)get_be(p, 8);
        case WF_NC_UINT64: return (double)get_be(p, 8);
        case WF_NC_FLOAT: {
            const uint32_t b = (uint32_t)get_be(p, 4);
            float x;
            std::memcpy(&x, &b, 4);
            return (double)x;
        }
        case WF_NC_DOUBLE: {
            const uint64_t b = get_be(p, 8);
            double x;
            std::memcpy(&x, &b, 8);
            return x;
        }
        default: return 0.0;
    }
}

// Encode x as type t; false when x does not fit an integer type.
bool encode_value(uint8_t* p, int32_t t, double x) {
    if (t == WF_NC_FLOAT) {
        const float y = (float)x;
        uint32_t b;
        std::memcpy(&b, &y, 4);
        put_be(p, b, 4);
        return true;
    }
    if (t == WF_NC_DOUBLE) {
        uint64_t b;
        std::memcpy(&b, &x, 8);
        put_be(p, b, 8);
        return true;
    }
    if (!(x == x)) return false;
    const double r = std::nearbyint(x);
    double lo, hi;
    switch (t) {
        case WF_NC_BYTE: lo = -128.0; hi = 127.0; break;
        case WF_NC_CHAR: case WF_NC_UBYTE: lo = 0.0; hi = 255.0; break;
        case WF_NC_SHORT: lo = -32768.0; hi = 32767.0; break;
        case WF_NC_USHORT: lo = 0.0; hi = 65535.0; break;
        case WF_NC_INT: lo = -2147483648.0; hi = 2147483647.0; break;
        case WF_NC_UINT: lo = 0.0; hi = 4294967295.0; break;
        case WF_NC_INT64: lo = -9223372036854775808.0; hi = 9223372036854774784.0; break;
        case WF_NC_UINT64: lo = 0.0; hi = 18446744073709549568.0; break;
        default: return false;
    }
    if (r < lo || r > hi) return false;
    const int n = type_size(t);
    if (t == WF_NC_UINT64) put_be(p, (uint64_t)r, n);
    else put_be(p, (uint64_t)(int64_t)r, n);
    return true;
}

struct NcAtt {
    std::string name;
    int32_t type = 0;
    int64_t n = 0;
    std::vector<uint8_t> raw;  // n values, big-endian, unpadded
};

struct NcVar {
    std::string name;
    std::vector<int32_t> dimids;
    std::vector<NcAtt> atts;
    int32_t type = 0;
    int64_t vsize = 0;  // padded size of one record (record variable) or of the whole variable
    int64_t begin = 0;
    bool record = false;
};

struct NcDim {
    std::string name;
    int64_t len = 0;  // 0 = record dimension
};

const NcAtt* find_att(const std::vector<NcAtt>& a, const char* name) {
    for (const auto& x : a)
        if (x.name == name) return &x;
    return nullptr;
}

}  // namespace

struct WfNcFile {
    FILE* fp = nullptr;
    bool writable = false;
    bool define_mode = false;
    int version = 1;
    int64_t numrecs = 0;
    int64_t recsize = 0;
    std::vector<NcDim> dims;
    std::vector<NcAtt> gatts;
    std::vector<NcVar> vars;
    std::string err;
};

namespace {

int fail(WfNcFile* f, int code, const std::string& msg) {
    if (f) f->err = msg;
    else g_nc_error = msg;
    return code;
}

// ---- header reading
struct HdrReader {
    FILE* fp;
    bool ok = true;
    uint64_t be(int n) {
        uint8_t b[8];
        if (std::fread(b, 1, n, fp) != (size_t)n) {
            ok = false;
            return 0;
        }
        return get_be(b, n);
    }
    std::string name(int cnt_bytes) {
        const uint64_t n = be(cnt_bytes);
        if (!ok || n > (1u << 20)) {
            ok = false;
            return {};
        }
        std::string s((size_t)n, '\0');
        if (n && std::fread(&s[0], 1, n, fp) != n) ok = false;
        skip(pad4((int64_t)n) - (int64_t)n);
        return s;
    }
    void skip(int64_t n) {
        uint8_t b[4];
        if (n > 0 && std::fread(b, 1, (size_t)n, fp) != (size_t)n) ok = false;
    }
};

bool read_atts(HdrReader& r, int cb, std::vector<NcAtt>& out) {
    const uint32_t tag = (uint32_t)r.be(4);
    const uint64_t n = r.be(cb);
    if (!r.ok) return false;
    if (tag == 0 && n == 0) return true;
    if (tag != TAG_ATTRIBUTE || n > (1u << 20)) return false;
    for (uint64_t i = 0; i < n && r.ok; ++i) {
        NcAtt a;
        a.name = r.name(cb);
        a.type = (int32_t)r.be(4);
        a.n = (int64_t)r.be(cb);
        const int ts = type_size(a.type);
        if (!ts || a.n < 0 || a.n > (1 << 26)) return false;
        a.raw.resize((size_t)(a.n * ts));
        if (!a.raw.empty() && std::fread(a.raw.data(), 1, a.raw.size(), r.fp) != a.raw.size()) return false;
        r.skip(pad4(a.n * ts) - a.n * ts);
        out.push_back(std::move(a));
    }
    return r.ok;
}

int read_header(WfNcFile* f) {
    HdrReader r{f->fp, true};
    char magic[4];
    if (std::fread(magic, 1, 4, f->fp) != 4 || magic[0] != 'C' || magic[1] != 'D' || magic[2] != 'F')
        return fail(f, WF_ERR_INVALID, "not a netCDF classic-format file (netCDF-4/HDF5 files must be converted)");
    f->version = magic[3];
    if (f->version != 1 && f->version != 2 && f->version != 5)
        return fail(f, WF_ERR_UNSUPPORTED, "unknown netCDF format version");
    const int cb = f->version == 5 ? 8 : 4;       // counts, lengths, ids, sizes
    const int ob = f->version == 1 ? 4 : 8;       // data offsets
    const uint64_t nrec = r.be(cb);
    const bool streaming = (cb == 4 && nrec == 0xffffffffull) || (cb == 8 && nrec == ~0ull);
    f->numrecs = streaming ? -1 : (int64_t)nrec;
    // dimensions
    {
        const uint32_t tag = (uint32_t)r.be(4);
        const uint64_t n = r.be(cb);
        if (!r.ok || !((tag == 0 && n == 0) || (tag == TAG_DIMENSION && n < (1u << 20))))
            return fail(f, WF_ERR_INVALID, "corrupt dimension list");
        for (uint64_t i = 0; i < n && r.ok; ++i) {
            NcDim d;
            d.name = r.name(cb);
            d.len = (int64_t)r.be(cb);
            f->dims.push_back(d);
        }
    }
    if (!read_atts(r, cb, f->gatts)) return fail(f, WF_ERR_INVALID, "corrupt global attribute list");
    {
        const uint32_t tag = (uint32_t)r.be(4);
        const uint64_t n = r.be(cb);
        if (!r.ok || !((tag == 0 && n == 0) || (tag == TAG_VARIABLE && n < (1u << 20))))
            return fail(f, WF_ERR_INVALID, "corrupt variable list");
        for (uint64_t i = 0; i < n && r.ok; ++i) {
            NcVar v;
            v.name = r.name(cb);
            const uint64_t nd = r.be(cb);
            if (nd > kMaxDims) return fail(f, WF_ERR_UNSUPPORTED, "variable with more than 16 dimensions");
            for (uint64_t k = 0; k < nd; ++k) {
                const uint64_t id = r.be(cb);
                if (id >= f->dims.size()) return fail(f, WF_ERR_INVALID, "dimension id out of range");
                v.dimids.push_back((int32_t)id);
            }
            if (!read_atts(r, cb, v.atts)) return fail(f, WF_ERR_INVALID, "corrupt variable attribute list");
            v.type = (int32_t)r.be(4);
            v.vsize = (int64_t)r.be(cb);
            v.begin = (int64_t)r.be(ob);
            if (!type_size(v.type)) return fail(f, WF_ERR_INVALID, "unknown variable type");
            for (size_t k = 0; k < v.dimids.size(); ++k)
                if (f->dims[v.dimids[k]].len == 0) {
                    if (k != 0) return fail(f, WF_ERR_INVALID, "record dimension not first");
                    v.record = true;
                }
            f->vars.push_back(std::move(v));
        }
    }
    if (!r.ok) return fail(f, WF_ERR_INVALID, "truncated header");
    // record size from the shapes (the header's vsize of a lone record variable may be padded)
    int nrecvars = 0;
    int64_t rs = 0;
    for (const auto& v : f->vars) {
        if (!v.record) continue;
        int64_t sz = type_size(v.type);
        for (size_t k = 1; k < v.dimids.size(); ++k) sz *= f->dims[v.dimids[k]].len;
        rs += pad4(sz);
        ++nrecvars;
        if (nrecvars == 1) f->recsize = sz;
    }
    if (nrecvars != 1) f->recsize = rs;
    if (f->numrecs < 0) {  // streaming: records from the file size
        f->numrecs = 0;
        int64_t rec_begin = -1;
        for (const auto& v : f->vars)
            if (v.record && (rec_begin < 0 || v.begin < rec_begin)) rec_begin = v.begin;
        if (rec_begin >= 0 && f->recsize > 0 && fseeko(f->fp, 0, SEEK_END) == 0) {
            const int64_t end = (int64_t)ftello(f->fp);
            f->numrecs = std::max<int64_t>(0, (end - rec_begin) / f->recsize);
        }
    }
    return WF_OK;
}

// Byte offset of element idx (C order over the variable's dimensions) and the length of the
// contiguous run along the last dimension starting there.
int64_t elem_offset(const WfNcFile* f, const NcVar& v, const int64_t* idx) {
    const int ts = type_size(v.type);
    const size_t nd = v.dimids.size();
    int64_t off = 0, stride = ts;
    for (size_t k = nd; k-- > (v.record ? 1 : 0);) {
        off += idx[k] * stride;
        stride *= f->dims[v.dimids[k]].len;
    }
    if (v.record) off += idx[0] * f->recsize;
    return v.begin + off;
}

// Walk the hyperslab in C order, calling fn(byte offset, first element index in the slab,
// run length) for each contiguous run along the last dimension.
template <class Fn>
bool for_runs(const WfNcFile* f, const NcVar& v, const int64_t* start, const int64_t* count, Fn fn) {
    const size_t nd = v.dimids.size();
    if (nd == 0) return fn(v.begin, (int64_t)0, (int64_t)1);
    if (v.record && nd == 1) {  // one value per record: records are recsize apart, not contiguous
        int64_t idx[1];
        for (int64_t r = 0; r < count[0]; ++r) {
            idx[0] = start[0] + r;
            if (!fn(elem_offset(f, v, idx), r, (int64_t)1)) return false;
        }
        return true;
    }
    int64_t idx[kMaxDims];
    for (size_t k = 0; k < nd; ++k) {
        if (count[k] == 0) return true;
        idx[k] = start[k];
    }
    const int64_t run = count[nd - 1];
    int64_t done = 0;
    while (true) {
        if (!fn(elem_offset(f, v, idx), done, run)) return false;
        done += run;
        size_t k = nd - 1;
        while (true) {
            if (k == 0) return true;
            --k;
            if (++idx[k] < start[k] + count[k]) break;
            idx[k] = start[k];
        }
    }
}

int check_slab(WfNcFile* f, const NcVar& v, const int64_t* start, const int64_t* count, bool writing) {
    for (size_t k = 0; k < v.dimids.size(); ++k) {
        const NcDim& d = f->dims[v.dimids[k]];
        const int64_t len = d.len == 0 ? (writing ? std::numeric_limits<int64_t>::max() / 2 : f->numrecs) : d.len;
        if (start[k] < 0 || count[k] < 0 || start[k] + count[k] > len)
            return fail(f, WF_ERR_INVALID, "hyperslab out of range for variable " + v.name);
    }
    return WF_OK;
}

void fill_record_range(WfNcFile* f, int64_t r0, int64_t r1);

// ---- header writing
struct HdrWriter {
    std::vector<uint8_t> b;
    void be(uint64_t v, int n) {
        uint8_t t[8];
        put_be(t, v, n);
        b.insert(b.end(), t, t + n);
    }
    void name(const std::string& s, int cb) {
        be(s.size(), cb);
        b.insert(b.end(), s.begin(), s.end());
        b.resize(b.size() + (size_t)(pad4((int64_t)s.size()) - (int64_t)s.size()), 0);
    }
    void atts(const std::vector<NcAtt>& a, int cb) {
        if (a.empty()) {
            be(0, 4);
            be(0, cb);
            return;
        }
        be(TAG_ATTRIBUTE, 4);
        be(a.size(), cb);
        for (const auto& x : a) {
            name(x.name, cb);
            be((uint32_t)x.type, 4);
            be((uint64_t)x.n, cb);
            b.insert(b.end(), x.raw.begin(), x.raw.end());
            b.resize(b.size() + (size_t)(pad4((int64_t)x.raw.size()) - (int64_t)x.raw.size()), 0);
        }
    }
};

std::vector<uint8_t> encode_header(const WfNcFile* f) {
    const int cb = f->version == 5 ? 8 : 4;
    const int ob = f->version == 1 ? 4 : 8;
    HdrWriter w;
    w.b = {'C', 'D', 'F', (uint8_t)f->version};
    w.be((uint64_t)f->numrecs, cb);
    if (f->dims.empty()) {
        w.be(0, 4);
        w.be(0, cb);
    } else {
        w.be(TAG_DIMENSION, 4);
        w.be(f->dims.size(), cb);
        for (const auto& d : f->dims) {
            w.name(d.name, cb);
            w.be((uint64_t)d.len, cb);
        }
    }
    w.atts(f->gatts, cb);
    if (f->vars.empty()) {
        w.be(0, 4);
        w.be(0, cb);
    } else {
        w.be(TAG_VARIABLE, 4);
        w.be(f->vars.size(), cb);
        for (const auto& v : f->vars) {
            w.name(v.name, cb);
            w.be(v.dimids.size(), cb);
            for (int32_t id : v.dimids) w.be((uint64_t)id, cb);
            w.atts(v.atts, cb);
            w.be((uint32_t)v.type, 4);
            const int64_t vs = (cb == 4 && v.vsize > 0xfffffffcLL) ? 0xffffffffLL : v.vsize;
            w.be((uint64_t)vs, cb);
            w.be((uint64_t)v.begin, ob);
        }
    }
    return w.b;
}

// the fill value of a variable (its _FillValue attribute, or the type's default)
double var_fill(const NcVar& v) {
    const NcAtt* a = find_att(v.atts, "_FillValue");
    if (a && a->n >= 1 && a->type == v.type) return decode_value(a->raw.data(), a->type);
    return default_fill(v.type);
}

bool write_at(WfNcFile* f, int64_t off, const uint8_t* p, size_t n) {
    return fseeko(f->fp, (off_t)off, SEEK_SET) == 0 && std::fwrite(p, 1, n, f->fp) == n;
}

// Fill value bytes of n elements of type t
std::vector<uint8_t> fill_bytes(const NcVar& v, int64_t n) {
    const int ts = type_size(v.type);
    std::vector<uint8_t> one(ts);
    if (!encode_value(one.data(), v.type, var_fill(v))) std::fill(one.begin(), one.end(), 0);
    std::vector<uint8_t> out((size_t)(n * ts));
    for (int64_t i = 0; i < n; ++i) std::memcpy(out.data() + i * ts, one.data(), ts);
    return out;
}

// Fill values of records [r0, r1) of every record variable, with each variable's padding (none
// for a lone record variable, whose records are not padded), so the file always ends on a whole
// record.
void fill_record_range(WfNcFile* f, int64_t r0, int64_t r1) {
    int nrec = 0;
    for (const auto& v : f->vars) nrec += v.record ? 1 : 0;
    for (const auto& v : f->vars) {
        if (!v.record) continue;
        int64_t n = 1;
        for (size_t k = 1; k < v.dimids.size(); ++k) n *= f->dims[v.dimids[k]].len;
        auto bytes = fill_bytes(v, n);
        if (nrec > 1) bytes.resize((size_t)v.vsize, 0);
        for (int64_t r = r0; r < r1; ++r) write_at(f, v.begin + r * f->recsize, bytes.data(), bytes.size());
    }
}

}  // namespace

extern "C" {

const char* wf_nc_last_error(const WfNcFile* f) { return f ? f->err.c_str() : g_nc_error.c_str(); }

int32_t wf_nc_open(const char* path, WfNcFile** out) {
    if (!out || !path) return fail(nullptr, WF_ERR_INVALID, "null argument");
    *out = nullptr;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(nullptr, WF_ERR_INVALID, std::string("cannot open ") + path);
    WfNcFile* f = new WfNcFile();
    f->fp = fp;
    const int rc = read_header(f);
    if (rc != WF_OK) {
        g_nc_error = f->err;
        wf_nc_close(f);
        return rc;
    }
    *out = f;
    return WF_OK;
}

void wf_nc_close(WfNcFile* f) {
    if (!f) return;
    if (f->fp) {
        if (f->writable && !f->define_mode) {  // the final number of records
            const int cb = f->version == 5 ? 8 : 4;
            uint8_t b[8];
            put_be(b, (uint64_t)f->numrecs, cb);
            write_at(f, 4, b, cb);
        }
        std::fclose(f->fp);
    }
    delete f;
}

int32_t wf_nc_format(const WfNcFile* f) { return f ? f->version : WF_ERR_INVALID; }
int64_t wf_nc_numrecs(const WfNcFile* f) { return f ? f->numrecs : (int64_t)WF_ERR_INVALID; }
int32_t wf_nc_ndims(const WfNcFile* f) { return f ? (int32_t)f->dims.size() : WF_ERR_INVALID; }
int32_t wf_nc_nvars(const WfNcFile* f) { return f ? (int32_t)f->vars.size() : WF_ERR_INVALID; }

static void copy_name(const std::string& s, char* dst, int32_t cap) {
    if (!dst || cap <= 0) return;
    const size_t n = std::min<size_t>(s.size(), (size_t)cap - 1);
    std::memcpy(dst, s.data(), n);
    dst[n] = '\0';
}

int32_t wf_nc_dim(const WfNcFile* f, int32_t i, char* name, int32_t cap, int64_t* len, int32_t* is_record) {
    if (!f || i < 0 || i >= (int32_t)f->dims.size()) return WF_ERR_INVALID;
    copy_name(f->dims[i].name, name, cap);
    if (len) *len = f->dims[i].len == 0 ? f->numrecs : f->dims[i].len;
    if (is_record) *is_record = f->dims[i].len == 0;
    return WF_OK;
}

int32_t wf_nc_var(const WfNcFile* f, int32_t i, char* name, int32_t cap, int32_t* type, int32_t* ndims,
                  int32_t* dimids) {
    if (!f || i < 0 || i >= (int32_t)f->vars.size()) return WF_ERR_INVALID;
    const NcVar& v = f->vars[i];
    copy_name(v.name, name, cap);
    if (type) *type = v.type;
    if (ndims) *ndims = (int32_t)v.dimids.size();
    if (dimids)
        for (size_t k = 0; k < v.dimids.size(); ++k) dimids[k] = v.dimids[k];
    return WF_OK;
}

int32_t wf_nc_varid(const WfNcFile* f, const char* name) {
    if (!f || !name) return -1;
    for (size_t i = 0; i < f->vars.size(); ++i)
        if (f->vars[i].name == name) return (int32_t)i;
    return -1;
}

static const std::vector<NcAtt>* att_list(const WfNcFile* f, int32_t varid) {
    if (!f) return nullptr;
    if (varid == WF_NC_GLOBAL) return &f->gatts;
    if (varid < 0 || varid >= (int32_t)f->vars.size()) return nullptr;
    return &f->vars[varid].atts;
}

int32_t wf_nc_natts(const WfNcFile* f, int32_t varid) {
    const auto* L = att_list(f, varid);
    return L ? (int32_t)L->size() : WF_ERR_INVALID;
}

int32_t wf_nc_att_name(const WfNcFile* f, int32_t varid, int32_t i, char* name, int32_t cap) {
    const auto* L = att_list(f, varid);
    if (!L || i < 0 || i >= (int32_t)L->size()) return WF_ERR_INVALID;
    copy_name((*L)[i].name, name, cap);
    return WF_OK;
}

int32_t wf_nc_att(const WfNcFile* f, int32_t varid, const char* name, int32_t* type, int64_t* n) {
    const auto* L = att_list(f, varid);
    const NcAtt* a = L ? find_att(*L, name) : nullptr;
    if (!a) return WF_ERR_INVALID;
    if (type) *type = a->type;
    if (n) *n = a->n;
    return WF_OK;
}

int32_t wf_nc_att_get(const WfNcFile* f, int32_t varid, const char* name, double* dst, int64_t cap) {
    const auto* L = att_list(f, varid);
    const NcAtt* a = L ? find_att(*L, name) : nullptr;
    if (!a || !dst) return WF_ERR_INVALID;
    const int ts = type_size(a->type);
    for (int64_t i = 0; i < a->n && i < cap; ++i) dst[i] = decode_value(a->raw.data() + i * ts, a->type);
    return WF_OK;
}

int32_t wf_nc_att_text(const WfNcFile* f, int32_t varid, const char* name, char* dst, int64_t cap) {
    const auto* L = att_list(f, varid);
    const NcAtt* a = L ? find_att(*L, name) : nullptr;
    if (!a || !dst || cap <= 0 || a->type != WF_NC_CHAR) return WF_ERR_INVALID;
    const int64_t n = std::min<int64_t>(a->n, cap - 1);
    if (n > 0) std::memcpy(dst, a->raw.data(), (size_t)n);
    dst[n] = '\0';
    return WF_OK;
}

int32_t wf_nc_get(WfNcFile* f, int32_t varid, const int64_t* start, const int64_t* count, double* dst,
                  int32_t decode) {
    if (!f || !dst || varid < 0 || varid >= (int32_t)f->vars.size()) return fail(f, WF_ERR_INVALID, "bad variable");
    if (f->define_mode) return fail(f, WF_ERR_INVALID, "file in define mode");
    const NcVar& v = f->vars[varid];
    const size_t nd = v.dimids.size();
    int64_t zero[kMaxDims] = {0}, one[kMaxDims];
    for (size_t k = 0; k < nd; ++k) one[k] = 1;
    if (nd > 0 && (!start || !count)) return fail(f, WF_ERR_INVALID, "start and count required");
    const int64_t* st = nd ? start : zero;
    const int64_t* ct = nd ? count : one;
    int rc = check_slab(f, v, st, ct, false);
    if (rc) return rc;
    const int ts = type_size(v.type);
    std::vector<uint8_t> buf;
    const bool ok = for_runs(f, v, st, ct, [&](int64_t off, int64_t at, int64_t n) {
        buf.resize((size_t)(n * ts));
        if (fseeko(f->fp, (off_t)off, SEEK_SET) != 0 || std::fread(buf.data(), 1, buf.size(), f->fp) != buf.size())
            return false;
        for (int64_t i = 0; i < n; ++i) dst[at + i] = decode_value(buf.data() + i * ts, v.type);
        return true;
    });
    if (!ok) return fail(f, WF_ERR_INVALID, "read past the end of the file for variable " + v.name);
    if (decode) {
        int64_t total = 1;
        for (size_t k = 0; k < nd; ++k) total *= ct[k];
        double fillv = 0.0, missv = 0.0, scale = 1.0, offset = 0.0;
        const bool has_fill = find_att(v.atts, "_FillValue") != nullptr;
        const bool has_miss = find_att(v.atts, "missing_value") != nullptr;
        const bool has_scale = find_att(v.atts, "scale_factor") != nullptr;
        const bool has_offset = find_att(v.atts, "add_offset") != nullptr;
        if (has_fill) wf_nc_att_get(f, varid, "_FillValue", &fillv, 1);
        if (has_miss) wf_nc_att_get(f, varid, "missing_value", &missv, 1);
        if (has_scale) wf_nc_att_get(f, varid, "scale_factor", &scale, 1);
        if (has_offset) wf_nc_att_get(f, varid, "add_offset", &offset, 1);
        const double NaN = std::numeric_limits<double>::quiet_NaN();
        for (int64_t i = 0; i < total; ++i) {
            double x = dst[i];
            if ((has_fill && x == fillv) || (has_miss && x == missv)) {
                dst[i] = NaN;
                continue;
            }
            if (has_scale) x = x * scale;
            if (has_offset) x = x + offset;
            dst[i] = x;
        }
    }
    return WF_OK;
}

int32_t wf_nc_create(const char* path, int32_t format, WfNcFile** out) {
    if (!out || !path) return fail(nullptr, WF_ERR_INVALID, "null argument");
    *out = nullptr;
    if (format != 1 && format != 2 && format != 5) return fail(nullptr, WF_ERR_INVALID, "format must be 1, 2 or 5");
    FILE* fp = std::fopen(path, "w+b");
    if (!fp) return fail(nullptr, WF_ERR_INVALID, std::string("cannot create ") + path);
    WfNcFile* f = new WfNcFile();
    f->fp = fp;
    f->writable = true;
    f->define_mode = true;
    f->version = format;
    *out = f;
    return WF_OK;
}

int32_t wf_nc_def_dim(WfNcFile* f, const char* name, int64_t len) {
    if (!f || !f->define_mode || !name || !*name || len < 0) return fail(f, WF_ERR_INVALID, "bad dimension");
    for (const auto& d : f->dims) {
        if (d.name == name) return fail(f, WF_ERR_INVALID, std::string("dimension exists: ") + name);
        if (len == 0 && d.len == 0) return fail(f, WF_ERR_INVALID, "only one record dimension");
    }
    if (f->version != 5 && len > 0xffffffffLL) return fail(f, WF_ERR_INVALID, "dimension too long for CDF-1/2");
    f->dims.push_back({name, len});
    return (int32_t)f->dims.size() - 1;
}

int32_t wf_nc_def_var(WfNcFile* f, const char* name, int32_t type, int32_t ndims, const int32_t* dimids) {
    if (!f || !f->define_mode || !name || !*name) return fail(f, WF_ERR_INVALID, "bad variable");
    if (!type_size(type) || (f->version != 5 && type > WF_NC_DOUBLE))
        return fail(f, WF_ERR_INVALID, "type not available in this format");
    if (ndims < 0 || ndims > kMaxDims || (ndims > 0 && !dimids)) return fail(f, WF_ERR_INVALID, "bad dimensions");
    if (wf_nc_varid(f, name) >= 0) return fail(f, WF_ERR_INVALID, std::string("variable exists: ") + name);
    NcVar v;
    v.name = name;
    v.type = type;
    for (int k = 0; k < ndims; ++k) {
        if (dimids[k] < 0 || dimids[k] >= (int32_t)f->dims.size()) return fail(f, WF_ERR_INVALID, "bad dimension id");
        if (f->dims[dimids[k]].len == 0) {
            if (k != 0) return fail(f, WF_ERR_INVALID, "the record dimension must come first");
            v.record = true;
        }
        v.dimids.push_back(dimids[k]);
    }
    f->vars.push_back(std::move(v));
    return (int32_t)f->vars.size() - 1;
}

static std::vector<NcAtt>* att_list_w(WfNcFile* f, int32_t varid) {
    if (!f || !f->define_mode) return nullptr;
    if (varid == WF_NC_GLOBAL) return &f->gatts;
    if (varid < 0 || varid >= (int32_t)f->vars.size()) return nullptr;
    return &f->vars[varid].atts;
}

static void set_att(std::vector<NcAtt>& L, NcAtt&& a) {
    for (auto& x : L)
        if (x.name == a.name) {
            x = std::move(a);
            return;
        }
    L.push_back(std::move(a));
}

int32_t wf_nc_put_att_text(WfNcFile* f, int32_t varid, const char* name, const char* text) {
    auto* L = att_list_w(f, varid);
    if (!L || !name || !*name || !text) return fail(f, WF_ERR_INVALID, "bad attribute");
    NcAtt a;
    a.name = name;
    a.type = WF_NC_CHAR;
    a.n = (int64_t)std::strlen(text);
    a.raw.assign(text, text + a.n);
    set_att(*L, std::move(a));
    return WF_OK;
}

int32_t wf_nc_put_att(WfNcFile* f, int32_t varid, const char* name, int32_t type, const double* values, int64_t n) {
    auto* L = att_list_w(f, varid);
    if (!L || !name || !*name || n < 0 || (n > 0 && !values) || !type_size(type) || type == WF_NC_CHAR ||
        (f->version != 5 && type > WF_NC_DOUBLE))
        return fail(f, WF_ERR_INVALID, "bad attribute");
    NcAtt a;
    a.name = name;
    a.type = type;
    a.n = n;
    const int ts = type_size(type);
    a.raw.resize((size_t)(n * ts));
    for (int64_t i = 0; i < n; ++i)
        if (!encode_value(a.raw.data() + i * ts, type, values[i]))
            return fail(f, WF_ERR_INVALID, std::string("attribute value out of range: ") + name);
    set_att(*L, std::move(a));
    return WF_OK;
}

int32_t wf_nc_enddef(WfNcFile* f) {
    if (!f || !f->define_mode) return fail(f, WF_ERR_INVALID, "not in define mode");
    // sizes
    int nrecvars = 0;
    int64_t lone = 0;
    for (auto& v : f->vars) {
        int64_t sz = type_size(v.type);
        for (size_t k = v.record ? 1 : 0; k < v.dimids.size(); ++k) sz *= f->dims[v.dimids[k]].len;
        v.vsize = pad4(sz);
        if (v.record) {
            ++nrecvars;
            lone = sz;
        }
    }
    // offsets: header, fixed-size variables, then the records
    int64_t off = (int64_t)encode_header(f).size();  // begins do not change the header size
    for (auto& v : f->vars)
        if (!v.record) {
            v.begin = off;
            off += v.vsize;
        }
    int64_t rs = 0;
    for (auto& v : f->vars)
        if (v.record) {
            v.begin = off + rs;
            rs += v.vsize;
        }
    f->recsize = nrecvars == 1 ? lone : rs;
    if (f->version == 1 && off + rs > 0x7fffffffLL) return fail(f, WF_ERR_INVALID, "data too large for CDF-1");
    const auto hdr = encode_header(f);
    if (!write_at(f, 0, hdr.data(), hdr.size())) return fail(f, WF_ERR_INVALID, "write failed");
    for (const auto& v : f->vars) {
        if (v.record) continue;
        int64_t n = 1;
        for (int32_t id : v.dimids) n *= f->dims[id].len;
        auto bytes = fill_bytes(v, n);
        bytes.resize((size_t)v.vsize, 0);
        if (!write_at(f, v.begin, bytes.data(), bytes.size())) return fail(f, WF_ERR_INVALID, "write failed");
    }
    f->define_mode = false;
    std::fflush(f->fp);
    return WF_OK;
}

int32_t wf_nc_put(WfNcFile* f, int32_t varid, const int64_t* start, const int64_t* count, const double* src) {
    if (!f || !f->writable || f->define_mode || !src || varid < 0 || varid >= (int32_t)f->vars.size())
        return fail(f, WF_ERR_INVALID, "bad write");
    const NcVar& v = f->vars[varid];
    const size_t nd = v.dimids.size();
    int64_t zero[kMaxDims] = {0}, one[kMaxDims];
    for (size_t k = 0; k < nd; ++k) one[k] = 1;
    if (nd > 0 && (!start || !count)) return fail(f, WF_ERR_INVALID, "start and count required");
    const int64_t* st = nd ? start : zero;
    const int64_t* ct = nd ? count : one;
    int rc = check_slab(f, v, st, ct, true);
    if (rc) return rc;
    if (v.record && ct[0] > 0 && st[0] + ct[0] > f->numrecs) {  // new records, prefilled
        const int64_t old = f->numrecs;
        f->numrecs = st[0] + ct[0];
        fill_record_range(f, old, f->numrecs);
    }
    const int ts = type_size(v.type);
    const double fv = var_fill(v);
    std::vector<uint8_t> buf;
    bool range_ok = true;
    const bool ok = for_runs(f, v, st, ct, [&](int64_t off, int64_t at, int64_t n) {
        buf.resize((size_t)(n * ts));
        for (int64_t i = 0; i < n; ++i) {
            const double x = src[at + i];
            if (!encode_value(buf.data() + i * ts, v.type, x == x ? x : fv)) {
                range_ok = false;
                return false;
            }
        }
        return write_at(f, off, buf.data(), buf.size());
    });
    if (!range_ok) return fail(f, WF_ERR_INVALID, "value out of range of the type of " + v.name);
    if (!ok) return fail(f, WF_ERR_INVALID, "write failed");
    return WF_OK;
}

}  // extern "C"
