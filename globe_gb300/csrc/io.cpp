// io.cpp -- readers and writers of GLOBE's file formats (host C++).
//
// Record table: checkInputs + readInputData (PCGsolver.cpp:465-587).  The
// header names the columns; INDIV, PHENO and TIMES are found by name and
// every other column, in file order, is a covariate; TIMES becomes the last
// column of X.  (The reference writes covariate j of a row at column j-3,
// which equals this when the three named columns come first -- the only
// layout it reads correctly.)  IDs are parsed as numbers and truncated to
// int; individual index = ID - 1 and must lie in [0, N) with N the number of
// distinct IDs.  Lines that are empty are skipped; a token that does not
// parse is an error (the reference silently keeps the previous value).
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_set>
#include <vector>

#include "globe.h"

namespace {

void put_err(char* err, int errlen, const char* fmt, ...) {
    if (!err || errlen <= 0) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, (size_t)errlen, fmt, ap);
    va_end(ap);
}

bool next_line(FILE* f, std::string& line) {
    line.clear();
    int ch;
    bool any = false;
    while ((ch = fgetc(f)) != EOF) {
        any = true;
        if (ch == '\n') return true;
        line.push_back((char)ch);
    }
    return any;
}

void split(const std::string& s, std::vector<std::string>& out) {
    out.clear();
    size_t i = 0, n = s.size();
    while (i < n) {
        while (i < n && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r')) ++i;
        if (i >= n) break;
        size_t j = i;
        while (j < n && !(s[j] == ' ' || s[j] == '\t' || s[j] == '\r')) ++j;
        out.emplace_back(s.substr(i, j - i));
        i = j;
    }
}

bool blank(const std::string& s) {
    for (char c : s)
        if (!(c == ' ' || c == '\t' || c == '\r')) return false;
    return true;
}

}  // namespace

// no_time: INDIV and PHENO are required and every other column, in file order, is
// a covariate (the reduced model's readInputData, varCompEst_reducedModel_noTime.cpp:191-247);
// otherwise TIMES is required too and becomes the last column of X.
static int read_records(const char* path, bool no_time, int64_t* Nrec_out, int32_t* N_out, int32_t* p_out,
                        int32_t* indiv, double* X, double* y, char* err, int errlen) {
    if (!path || !Nrec_out || !N_out || !p_out) return GLOBE_ERR_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) {
        put_err(err, errlen, "Error opening input file: %s", path);
        return GLOBE_ERR_IO;
    }
    std::string line;
    std::vector<std::string> tok;
    if (!next_line(f, line)) {
        std::fclose(f);
        put_err(err, errlen, "empty input file: %s", path);
        return GLOBE_ERR_FORMAT;
    }
    split(line, tok);
    int ci = -1, cp = -1, ct = -1;
    for (int c = 0; c < (int)tok.size(); ++c) {
        if (tok[c] == "INDIV") ci = c;
        else if (tok[c] == "PHENO") cp = c;
        else if (tok[c] == "TIMES") ct = c;
    }
    if (no_time) ct = -1;   // a TIMES column, if any, is an ordinary covariate
    if (ci < 0 || cp < 0 || (!no_time && ct < 0)) {
        std::fclose(f);
        put_err(err, errlen, no_time ? "Missing required columns in header (INDIV, PHENO)."
                                     : "Missing required columns in header (INDIV, PHENO, TIMES).");
        return GLOBE_ERR_FORMAT;
    }
    const int ncol = (int)tok.size();
    const int p = ncol - (no_time ? 2 : 3);
    std::vector<int> covpos(ncol, -1);
    for (int c = 0, q = 0; c < ncol; ++c)
        if (c != ci && c != cp && c != ct) covpos[c] = q++;
    const bool fill = X != nullptr;
    const int64_t cap = fill ? *Nrec_out : 0;
    int64_t row = 0;
    std::unordered_set<int> ids;
    int lineno = 1;
    int rc = GLOBE_OK;
    std::vector<int> raw_ids;
    while (next_line(f, line)) {
        ++lineno;
        if (blank(line)) continue;
        split(line, tok);
        if ((int)tok.size() < ncol) {
            put_err(err, errlen, "line %d: %d fields, header has %d", lineno, (int)tok.size(), ncol);
            rc = GLOBE_ERR_FORMAT;
            break;
        }
        double v[512];
        std::vector<double> big;
        double* vals = v;
        if (ncol > 512) {
            big.resize(ncol);
            vals = big.data();
        }
        bool bad = false;
        for (int c = 0; c < ncol; ++c) {
            char* end = nullptr;
            errno = 0;
            vals[c] = std::strtod(tok[c].c_str(), &end);
            if (end == tok[c].c_str() || *end != '\0') {
                put_err(err, errlen, "line %d, column %d: cannot parse '%s'", lineno, c + 1, tok[c].c_str());
                bad = true;
                break;
            }
        }
        if (bad) {
            rc = GLOBE_ERR_FORMAT;
            break;
        }
        const int id = (int)vals[ci];  // (int) cast as in PCGsolver.cpp:511
        ids.insert(id);
        if (fill) {
            if (row >= cap) {
                put_err(err, errlen, "more records than on the first pass");
                rc = GLOBE_ERR_FORMAT;
                break;
            }
            raw_ids.push_back(id);
            y[row] = vals[cp];
            if (ct >= 0) X[(size_t)p * cap + row] = vals[ct];
            for (int c = 0; c < ncol; ++c)
                if (covpos[c] >= 0) X[(size_t)covpos[c] * cap + row] = vals[c];
        }
        ++row;
    }
    std::fclose(f);
    if (rc != GLOBE_OK) return rc;
    if (row == 0) {
        put_err(err, errlen, "no records in %s", path);
        return GLOBE_ERR_FORMAT;
    }
    const int N = (int)ids.size();
    if (fill) {
        if (row != cap) {
            put_err(err, errlen, "record count changed between passes");
            return GLOBE_ERR_FORMAT;
        }
        for (int64_t r = 0; r < row; ++r) {
            const int idx = raw_ids[r] - 1;
            if (idx < 0 || idx >= N) {
                put_err(err, errlen,
                        "record %lld: INDIV %d outside 1..%d (IDs must be 1..N in .fam order, N = number of "
                        "distinct IDs)", (long long)r + 1, raw_ids[r], N);
                return GLOBE_ERR_FORMAT;
            }
            if (indiv) indiv[r] = idx;
        }
    }
    *Nrec_out = row;
    *N_out = N;
    *p_out = p;
    return GLOBE_OK;
}

extern "C" int globe_read_records(const char* path, int64_t* Nrec_out, int32_t* N_out, int32_t* p_out,
                                  int32_t* indiv, double* X, double* y, char* err, int errlen) {
    return read_records(path, false, Nrec_out, N_out, p_out, indiv, X, y, err, errlen);
}

extern "C" int globe_read_records_no_time(const char* path, int64_t* Nrec_out, int32_t* N_out, int32_t* p_out,
                                          int32_t* indiv, double* X, double* y, char* err, int errlen) {
    return read_records(path, true, Nrec_out, N_out, p_out, indiv, X, y, err, errlen);
}

static int save_vec(const char* path, const void* payload, int32_t n, size_t esz) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return GLOBE_ERR_IO;
    bool ok = std::fwrite(&n, sizeof(int32_t), 1, f) == 1;
    if (n > 0) ok = ok && std::fwrite(payload, esz, (size_t)n, f) == (size_t)n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? GLOBE_OK : GLOBE_ERR_IO;
}

extern "C" int globe_save_vector_f32(const char* path, const double* v, int32_t n) {
    if (!path || n < 0 || (n > 0 && !v)) return GLOBE_ERR_ARG;
    std::vector<float> buf(n);
    for (int32_t i = 0; i < n; ++i) buf[i] = (float)v[i];
    return save_vec(path, buf.data(), n, sizeof(float));
}

extern "C" int globe_save_vector_f64(const char* path, const double* v, int32_t n) {
    if (!path || n < 0 || (n > 0 && !v)) return GLOBE_ERR_ARG;
    return save_vec(path, v, n, sizeof(double));
}

extern "C" int globe_bed_dims(const char* prefix, int32_t N, int64_t* M, char* err, int errlen) {
    if (!prefix || !M || N < 1) return GLOBE_ERR_ARG;
    std::string bim = std::string(prefix) + ".bim", bed = std::string(prefix) + ".bed";
    FILE* f = std::fopen(bim.c_str(), "rb");
    if (!f) {
        put_err(err, errlen, "Error opening .bim file: %s", bim.c_str());
        return GLOBE_ERR_IO;
    }
    int64_t lines = 0;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0)
        for (size_t i = 0; i < got; ++i) lines += buf[i] == '\n';
    std::fclose(f);
    f = std::fopen(bed.c_str(), "rb");
    if (!f) {
        put_err(err, errlen, "Error opening .bed file: %s", bed.c_str());
        return GLOBE_ERR_IO;
    }
    unsigned char magic[3] = {0, 0, 0};
    size_t nm = std::fread(magic, 1, 3, f);
    std::fclose(f);
    if (nm != 3 || magic[0] != 0x6C || magic[1] != 0x1B) {
        put_err(err, errlen, "Invalid .bed format (magic mismatch).");
        return GLOBE_ERR_FORMAT;
    }
    if (magic[2] == 0x00) {
        put_err(err, errlen, "BED is individual-major, code expects SNP-major.");
        return GLOBE_ERR_FORMAT;
    }
    if (magic[2] != 0x01) {
        put_err(err, errlen, "Third byte of .bed unknown.");
        return GLOBE_ERR_FORMAT;
    }
    struct stat st;
    if (stat(bed.c_str(), &st) != 0) {
        put_err(err, errlen, "cannot stat %s", bed.c_str());
        return GLOBE_ERR_IO;
    }
    const int64_t bps = ((int64_t)N + 3) / 4;
    if ((int64_t)st.st_size < 3 + lines * bps) {
        put_err(err, errlen, ".bed holds %lld bytes, need %lld for %lld SNPs x %d samples", (long long)st.st_size,
                (long long)(3 + lines * bps), (long long)lines, N);
        return GLOBE_ERR_FORMAT;
    }
    *M = lines;
    return GLOBE_OK;
}

extern "C" int globe_read_bed(const char* prefix, int32_t N, int64_t M, uint8_t* payload, char* err, int errlen) {
    if (!prefix || N < 1 || M < 0 || (M > 0 && !payload)) return GLOBE_ERR_ARG;
    std::string bed = std::string(prefix) + ".bed";
    FILE* f = std::fopen(bed.c_str(), "rb");
    if (!f) {
        put_err(err, errlen, "Error opening .bed file: %s", bed.c_str());
        return GLOBE_ERR_IO;
    }
    const size_t bytes = (size_t)M * (size_t)(((int64_t)N + 3) / 4);
    bool ok = std::fseek(f, 3, SEEK_SET) == 0;
    size_t got = 0;
    while (ok && got < bytes) {
        size_t r = std::fread(payload + got, 1, bytes - got, f);
        if (r == 0) break;
        got += r;
    }
    std::fclose(f);
    if (got != bytes) {
        put_err(err, errlen, "short read from %s", bed.c_str());
        return GLOBE_ERR_IO;
    }
    return GLOBE_OK;
}

extern "C" int globe_read_grm(const char* prefix, int32_t N, float* grm_lt, char* err, int errlen) {
    if (!prefix || N < 1 || !grm_lt) return GLOBE_ERR_ARG;
    std::string fn = std::string(prefix) + ".grm.bin";
    FILE* f = std::fopen(fn.c_str(), "rb");
    if (!f) {
        put_err(err, errlen, "Error opening GRM file: %s", fn.c_str());
        return GLOBE_ERR_IO;
    }
    const size_t nelt = (size_t)N * ((size_t)N + 1) / 2;
    size_t got = 0;
    while (got < nelt) {
        size_t r = std::fread(grm_lt + got, sizeof(float), nelt - got, f);
        if (r == 0) break;
        got += r;
    }
    std::fclose(f);
    if (got != nelt) {
        put_err(err, errlen, "Error reading from file: %s (%zu of %zu values)", fn.c_str(), got, nelt);
        return GLOBE_ERR_FORMAT;
    }
    return GLOBE_OK;
}

extern "C" int globe_write_grm(const char* prefix, const float* grm_lt, int32_t N, char* err, int errlen) {
    if (!prefix || N < 1 || !grm_lt) return GLOBE_ERR_ARG;
    std::string fn = std::string(prefix) + ".grm.bin";
    FILE* f = std::fopen(fn.c_str(), "wb");
    if (!f) {
        put_err(err, errlen, "Error opening %s for writing", fn.c_str());
        return GLOBE_ERR_IO;
    }
    const size_t nelt = (size_t)N * ((size_t)N + 1) / 2;
    size_t put = 0;
    while (put < nelt) {
        size_t w = std::fwrite(grm_lt + put, sizeof(float), std::min<size_t>(nelt - put, (size_t)1 << 26), f);
        if (w == 0) break;
        put += w;
    }
    const bool ok = put == nelt && std::fclose(f) == 0;
    if (put != nelt) std::fclose(f);
    if (!ok) {
        put_err(err, errlen, "Error writing %s (%zu of %zu values)", fn.c_str(), put, nelt);
        return GLOBE_ERR_IO;
    }
    return GLOBE_OK;
}
