// fair_io.cu -- file formats of the reference's driver (include/fair_io.h).
// Host code only.
//
// Matrix files: gfortran unformatted sequential records. A record is
// [int32 length][bytes][int32 length]; gfortran splits a record longer than
// 2147483639 bytes into subrecords whose leading marker is negative when more
// subrecords follow and whose trailing marker is negative when the subrecord
// continues an earlier one. Both machines here are little-endian, as the
// files of an x86 or aarch64 gfortran build are.
//
// Text files: Fortran list-directed READ. Every READ statement starts at the
// next line, takes its items from as many lines as it needs (separators:
// blanks, commas, tabs) and discards what is left of its last line; real
// numbers may use a D exponent.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fair_internal.cuh"
#include "fair_io.h"

namespace fair {
namespace {

constexpr int64_t kMaxSubrecord = 2147483639;

struct File {
    FILE *f = nullptr;
    explicit File(const char *path, const char *mode) { f = fopen(path, mode); }
    ~File() {
        if (f) fclose(f);
    }
};

int io_fail(const std::string &what) {
    set_detail(what);
    return FAIR_ERR_ARG;
}

int write_record(FILE *f, const void *data, int64_t bytes) {
    const char *p = static_cast<const char *>(data);
    int64_t left = bytes;
    bool first = true;
    do {
        const int64_t len = left > kMaxSubrecord ? kMaxSubrecord : left;
        const bool more = left > len;
        const int32_t head = more ? -(int32_t)len : (int32_t)len;
        const int32_t tail = first ? (int32_t)len : -(int32_t)len;
        if (fwrite(&head, 4, 1, f) != 1) return io_fail("write failed");
        if (len > 0 && fwrite(p, 1, (size_t)len, f) != (size_t)len) return io_fail("write failed");
        if (fwrite(&tail, 4, 1, f) != 1) return io_fail("write failed");
        p += len;
        left -= len;
        first = false;
    } while (left > 0);
    return FAIR_OK;
}

// Reads one record of exactly `bytes` bytes into out (NULL: skip it).
int read_record(FILE *f, void *out, int64_t bytes, const char *what) {
    char *p = static_cast<char *>(out);
    int64_t got = 0;
    for (;;) {
        int32_t head = 0, tail = 0;
        if (fread(&head, 4, 1, f) != 1) return io_fail(std::string("end of file reading ") + what);
        const int64_t len = head < 0 ? -(int64_t)head : head;
        if (got + len > bytes) return io_fail(std::string("record too long: ") + what);
        if (len > 0) {
            if (p) {
                if (fread(p + got, 1, (size_t)len, f) != (size_t)len)
                    return io_fail(std::string("end of file reading ") + what);
            } else if (fseeko(f, (off_t)len, SEEK_CUR) != 0) {
                return io_fail(std::string("end of file reading ") + what);
            }
        }
        if (fread(&tail, 4, 1, f) != 1) return io_fail(std::string("end of file reading ") + what);
        if ((tail < 0 ? -(int64_t)tail : tail) != len)
            return io_fail(std::string("record markers disagree: ") + what);
        got += len;
        if (head >= 0) break;
    }
    if (got != bytes) return io_fail(std::string("record too short: ") + what);
    return FAIR_OK;
}

int read_header(FILE *f, int32_t &m, int32_t &n, int32_t &nnz) {
    FAIR_TRY(read_record(f, &m, 4, "m"));
    FAIR_TRY(read_record(f, &n, 4, "n"));
    FAIR_TRY(read_record(f, &nnz, 4, "nnz"));
    if (m < 0 || n < 0 || nnz < 0) return io_fail("negative matrix sizes in the file");
    return FAIR_OK;
}

// ---- list-directed text ----------------------------------------------------------
struct ListReader {
    FILE *f;
    std::vector<std::string> pending;  // tokens left on the current line
    size_t pos = 0;
    bool eof = false;

    bool next_line() {
        std::string line;
        int c;
        bool any = false;
        while ((c = fgetc(f)) != EOF) {
            any = true;
            if (c == '\n') break;
            line.push_back((char)c);
        }
        if (!any) { eof = true; return false; }
        pending.clear();
        pos = 0;
        std::string tok;
        for (char ch : line) {
            if (ch == ' ' || ch == '\t' || ch == ',' || ch == '\r') {
                if (!tok.empty()) { pending.push_back(tok); tok.clear(); }
            } else {
                tok.push_back(ch);
            }
        }
        if (!tok.empty()) pending.push_back(tok);
        return true;
    }
    // One READ statement of k items.
    bool read(std::vector<std::string> &items, int k) {
        items.clear();
        if (!next_line()) return false;
        while ((int)items.size() < k) {
            if (pos < pending.size()) {
                items.push_back(pending[pos++]);
            } else if (!next_line()) {
                return false;
            }
        }
        return true;  // the rest of the line is dropped by the next READ
    }
};

bool to_double(std::string s, double &v) {
    for (char &c : s)
        if (c == 'd' || c == 'D') c = 'e';
    char *end = nullptr;
    errno = 0;
    v = strtod(s.c_str(), &end);
    return end && *end == '\0' && end != s.c_str();
}

bool to_int(const std::string &s, int64_t &v) {
    char *end = nullptr;
    errno = 0;
    long long t = strtoll(s.c_str(), &end, 10);
    if (!end || *end != '\0' || end == s.c_str() || errno) return false;
    v = t;
    return true;
}

// header of read_data: six "name value" READs (system_generation.f90:511-516)
struct DataHeader {
    int32_t n = 0, p = 0, nth = 0;
    double r = 0, dw = 0, sd = 0;
};

int read_data_header(ListReader &L, DataHeader &h) {
    std::vector<std::string> it;
    int64_t iv;
    const char *names[3] = {"n", "p", "nth"};
    int32_t *dst[3] = {&h.n, &h.p, &h.nth};
    for (int k = 0; k < 3; ++k) {
        if (!L.read(it, 2) || !to_int(it[1], iv) || iv < INT32_MIN || iv > INT32_MAX)
            return io_fail(std::string("cannot read ") + names[k]);
        *dst[k] = (int32_t)iv;
    }
    const char *rn[3] = {"r", "dw", "sd"};
    double *rd[3] = {&h.r, &h.dw, &h.sd};
    for (int k = 0; k < 3; ++k)
        if (!L.read(it, 2) || !to_double(it[1], *rd[k]))
            return io_fail(std::string("cannot read ") + rn[k]);
    return FAIR_OK;
}

}  // namespace
}  // namespace fair

using fair::io_fail;

extern "C" {

int fair_write_csr_file(const char *path, int32_t m, int32_t n, int32_t nnz, const double *vA,
                        const int32_t *JA, const int32_t *IA) {
    if (!path || !IA || (nnz > 0 && (!vA || !JA))) return FAIR_ERR_NULL;
    if (m < 0 || n < 0 || nnz < 0) return io_fail("negative matrix sizes");
    fair::File F(path, "wb");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    FAIR_TRY(fair::write_record(F.f, &m, 4));
    FAIR_TRY(fair::write_record(F.f, &n, 4));
    FAIR_TRY(fair::write_record(F.f, &nnz, 4));
    FAIR_TRY(fair::write_record(F.f, vA, 8 * (int64_t)nnz));
    FAIR_TRY(fair::write_record(F.f, JA, 4 * (int64_t)nnz));
    FAIR_TRY(fair::write_record(F.f, IA, 4 * ((int64_t)m + 1)));
    if (fflush(F.f) != 0) return io_fail("write failed");
    return FAIR_OK;
}

int fair_read_csr_file_sizes(const char *path, int32_t *m, int32_t *n, int32_t *nnz) {
    if (!path || !m || !n || !nnz) return FAIR_ERR_NULL;
    fair::File F(path, "rb");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    return fair::read_header(F.f, *m, *n, *nnz);
}

int fair_read_csr_file(const char *path, double *vA, int32_t *JA, int32_t *IA) {
    if (!path || !IA) return FAIR_ERR_NULL;
    fair::File F(path, "rb");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    int32_t m, n, nnz;
    FAIR_TRY(fair::read_header(F.f, m, n, nnz));
    if (nnz > 0 && (!vA || !JA)) return FAIR_ERR_NULL;
    FAIR_TRY(fair::read_record(F.f, vA, 8 * (int64_t)nnz, "vA"));
    FAIR_TRY(fair::read_record(F.f, JA, 4 * (int64_t)nnz, "JA"));
    FAIR_TRY(fair::read_record(F.f, IA, 4 * ((int64_t)m + 1), "IA"));
    return FAIR_OK;
}

int fair_store_matrix(fair_csr h, const char *path) {
    if (!h || !path) return FAIR_ERR_NULL;
    int32_t m = 0, n = 0;
    int64_t nnz = 0;
    FAIR_TRY(fair_csr_info(h, &m, &n, &nnz));
    if (nnz > INT32_MAX) return io_fail("nnz does not fit the file's 4-byte integers");
    std::vector<double> vA((size_t)nnz);
    std::vector<int64_t> IA((size_t)m + 1);
    std::vector<int32_t> JA((size_t)nnz), IA32((size_t)m + 1);
    FAIR_TRY(fair_csr_download(h, vA.data(), IA.data(), JA.data()));
    for (size_t i = 0; i < IA.size(); ++i) IA32[i] = (int32_t)IA[i];
    return fair_write_csr_file(path, m, n, (int32_t)nnz, vA.data(), JA.data(), IA32.data());
}

int fair_read_csr_matrix(fair_csr h, const char *path) {
    if (!h || !path) return FAIR_ERR_NULL;
    int32_t m, n, nnz;
    FAIR_TRY(fair_read_csr_file_sizes(path, &m, &n, &nnz));
    std::vector<double> vA((size_t)nnz + 1);
    std::vector<int32_t> JA((size_t)nnz + 1), IA((size_t)m + 1);
    FAIR_TRY(fair_read_csr_file(path, vA.data(), JA.data(), IA.data()));
    if (IA[0] != 0 || IA[m] != nnz) return io_fail("IA(0) must be 0 and IA(m) = nnz");
    return fair_construct_csr_matrix(m, n, vA.data(), IA.data(), JA.data(), h);
}

int fair_read_data_sizes(const char *path, int32_t *n, int32_t *p, int32_t *nth) {
    if (!path || !n || !p || !nth) return FAIR_ERR_NULL;
    fair::File F(path, "r");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    fair::ListReader L{F.f};
    fair::DataHeader hd;
    FAIR_TRY(fair::read_data_header(L, hd));
    *n = hd.n;
    *p = hd.p;
    *nth = hd.nth;
    return FAIR_OK;
}

int fair_read_data(const char *path, fair_data *dat, double *theta, double *T) {
    if (!path || !dat || !theta || !T) return FAIR_ERR_NULL;
    fair::File F(path, "r");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    fair::ListReader L{F.f};
    fair::DataHeader hd;
    FAIR_TRY(fair::read_data_header(L, hd));
    std::vector<std::string> it;
    int64_t l;
    // angles in degrees (:518-525)
    if (!L.read(it, 2) || !fair::to_int(it[1], l)) return io_fail("cannot read the angle count");
    if (l != hd.nth) return io_fail("Angle vector has the wrong length, nth is incorrect.");
    const double pi = 3.141592653589793;  // 4*atan(1d0)
    for (int64_t i = 0; i < l; ++i) {
        double v;
        if (!L.read(it, 1) || !fair::to_double(it[0], v)) return io_fail("cannot read an angle");
        theta[i] = v / 180.0 * pi;
    }
    // transmission data (:528-534)
    if (!L.read(it, 2) || !fair::to_int(it[1], l)) return io_fail("cannot read the data count");
    if (l != (int64_t)hd.nth * hd.p) return io_fail("Data has the wrong size, or p and nth are incorrect.");
    for (int64_t i = 0; i < l; ++i) {
        double v;
        if (!L.read(it, 1) || !fair::to_double(it[0], v)) return io_fail("cannot read a data value");
        T[i] = v;
    }
    dat->n = hd.n;
    dat->p = hd.p;
    dat->nth = hd.nth;
    dat->r = hd.r;
    dat->dw = hd.dw;
    dat->sd = hd.sd;
    dat->theta = theta;
    return FAIR_OK;
}

int fair_read_ordering(const char *path, int32_t *len, int32_t *order, int32_t capacity) {
    if (!path || !len) return FAIR_ERR_NULL;
    fair::File F(path, "r");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    fair::ListReader L{F.f};
    std::vector<std::string> it;
    int64_t l;
    if (!L.read(it, 2) || !fair::to_int(it[1], l) || l < 0 || l > INT32_MAX)
        return io_fail("cannot read the ordering length");
    *len = (int32_t)l;
    if (!order) return FAIR_OK;
    if (l > capacity) return io_fail("ordering longer than the buffer");
    for (int64_t i = 0; i < l; ++i) {
        int64_t v;
        if (!L.read(it, 1) || !fair::to_int(it[0], v)) return io_fail("cannot read an ordering entry");
        order[i] = (int32_t)v;
    }
    return FAIR_OK;
}

int fair_read_ref(const char *path, int64_t n, double *xref) {
    if (!path || !xref) return FAIR_ERR_NULL;
    fair::File F(path, "r");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    fair::ListReader L{F.f};
    std::vector<std::string> it;
    for (int64_t i = 0; i < n; ++i)
        if (!L.read(it, 1) || !fair::to_double(it[0], xref[i]))
            return io_fail("cannot read a reference value");
    return FAIR_OK;
}

int fair_write_values(const char *path, const double *x, int64_t n) {
    if (!path || (n > 0 && !x)) return FAIR_ERR_NULL;
    fair::File F(path, "w");
    if (!F.f) return io_fail(std::string("cannot open ") + path + ": " + strerror(errno));
    // list-directed REAL(8): G-style, 17 significant digits, width 25 after
    // the leading blank; F layout for 0.1 <= |x| < 1e17, else E with a
    // three-digit exponent
    char buf[64];
    for (int64_t k = 0; k < n; ++k) {
        const double v = x[k], a = fabs(v);
        if (std::isfinite(v) && (v == 0.0 || (a >= 0.1 && a < 1e17))) {
            // k: 10^(k-1) <= |v| < 10^k; 17 - k decimals; rounding can carry
            // |v| up to 10^k, one more integer digit
            int k = v == 0.0 ? 1 : (int)floor(log10(a)) + 1;
            if (v != 0.0 && k < 17) {
                char probe[64];
                snprintf(probe, sizeof probe, "%.*f", 17 - k, a);
                if (strtod(probe, nullptr) >= pow(10.0, k)) ++k;
            }
            const int dec = v == 0.0 ? 16 : (17 - k < 0 ? 0 : 17 - k);
            snprintf(buf, sizeof buf, "%.*f", dec, v);
            fprintf(F.f, " %20s     \n", buf);
        } else if (std::isfinite(v)) {
            snprintf(buf, sizeof buf, "%.16E", v);  // d.ddddE+xx
            // widen the exponent to three digits
            char *E = strchr(buf, 'E');
            int ex = atoi(E + 1);
            *E = '\0';
            fprintf(F.f, " %20sE%+04d\n", buf, ex);
        } else {
            fprintf(F.f, " %25s\n", std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
        }
    }
    if (fflush(F.f) != 0) return io_fail("write failed");
    return FAIR_OK;
}

}  // extern "C"
