// tbl_restart.cpp -- the reference's restart, counter and monitor files
// (host only).
//
// Tecplot ASCII POINT files, one record per grid point, i outermost, then j,
// then k, an empty record before every i block and every j block, three
// header records (title with time and nstep, variables, zone sizes):
//   TBL_TP_DNSTBL2   15 columns x y z U V W P Um Vm Wm Uf Vf Wf Wt Nk,
//                    FORMAT(3(1X,F10.6),11(1X,E22.15),(1X,I4))
//                    (dnstbl2/dnstbl.f90:2357-2384; read at :147-159, :350-358)
//   TBL_TP_ORIGINAL  8 columns x y z U V W T P, FORMAT(3(1X,F10.6),5(1X,E22.15))
//                    (originalTBL/fnldnstbl.f90:1696-1717, :2393)
//   TBL_TP_DNSSETBL  7 columns x y z U V W P, FORMAT(3(1X,F10.6),4(1X,E22.15))
//                    (dnssetbl/dnssetbl.f90:908-932; read at :119-134)
// A per-rank file holds j = 2..ny-1 and the rank's k range; the merged file
// that a run restarts from holds every j (the mergers dnstbl/restart.f90,
// originalTBL/restart.f90, dnssetbl/combineFile.f90).  The temperature column
// of the 8-column format is written as zero (the step has no temperature).
// Values carry 15 significant digits (E22.15), as in the reference, so a
// restart through these files is not bit-exact in FP64.
#include "../../include/tbl_gpu.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

int ncols(int format) { return format == TBL_TP_DNSTBL2 ? 15 : (format == TBL_TP_ORIGINAL ? 8 : 7); }
bool valid_format(int f) { return f == TBL_TP_DNSTBL2 || f == TBL_TP_ORIGINAL || f == TBL_TP_DNSSETBL; }

// Fortran Ew.d output: [-]0.<d digits>E+xx, right-justified in w columns,
// after one blank (the 1X before every field of the reference's formats).
// The d significant digits come from the correctly rounded %.*E conversion;
// the exponent is one more than C's (mantissa 0.d... instead of d.d...).  An
// exponent beyond two digits drops the E, as Ew.d does.
void put_e_wd(std::string& out, double v, int w, int d) {
    char buf[64], body[64];
    if (v == 0.0) {
        snprintf(body, sizeof body, "0.%0*dE+00", d, 0);
    } else if (!std::isfinite(v)) {
        snprintf(body, sizeof body, "%s", std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
    } else {
        snprintf(buf, sizeof buf, "%.*E", d - 1, std::fabs(v));  // d.ddd E+xx
        const char* e = strchr(buf, 'E');
        const int ex = atoi(e + 1) + 1;
        char digits[40];
        digits[0] = buf[0];
        memcpy(digits + 1, buf + 2, (size_t)(d - 1));
        digits[d] = 0;
        const char* sg = v < 0 ? "-" : "";
        if (ex > 99 || ex < -99)
            snprintf(body, sizeof body, "%s0.%s%c%03d", sg, digits, ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
        else
            snprintf(body, sizeof body, "%s0.%sE%c%02d", sg, digits, ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    }
    char field[80];
    snprintf(field, sizeof field, " %*s", w, body);
    out += field;
}

void put_e(std::string& out, double v) { put_e_wd(out, v, 22, 15); }

void put_f(std::string& out, double v, int w, int d) {
    char buf[64];
    snprintf(buf, sizeof buf, " %*.*f", w, d, v);
    out += buf;
}

// Fortran Fw.d output after nb blanks (the nX edit descriptor before the
// field): the value with d decimals right-justified in w columns, w asterisks
// when it needs more, NaN and Infinity spelled out.  C's %.*f rounds the
// exact binary value to nearest, as gfortran's F editing does, and keeps the
// minus sign of a negative value that rounds to zero, as gfortran does.
void put_fw(std::string& out, double v, int nb, int w, int d) {
    char body[400];
    if (std::isnan(v))
        snprintf(body, sizeof body, "NaN");
    else if (std::isinf(v))
        snprintf(body, sizeof body, "%s", w >= 9 ? (v > 0 ? "Infinity" : "-Infinity") : (v > 0 ? "Inf" : "-Inf"));
    else
        snprintf(body, sizeof body, "%.*f", d, v);
    out.append((size_t)nb, ' ');
    const int len = (int)strlen(body);
    if (len > w) {
        out.append((size_t)w, '*');
    } else {
        out.append((size_t)(w - len), ' ');
        out += body;
    }
}

// Fortran Ew.d output after nb blanks.
void put_ew(std::string& out, double v, int nb, int w, int d) {
    std::string f;
    put_e_wd(f, v, w, d);  // one blank, then the field
    out.append((size_t)nb, ' ');
    out.append(f, 1, std::string::npos);
}

inline size_t id3(int nx, int ny, int i, int j, int k) {  // 0-based
    return (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * (size_t)k);
}
inline double at3(const double* a, size_t p) { return a ? a[p] : 0.0; }

// Header records.  style 1: the program's own restart writer; style 2: the
// merger's (dnssetbl's combineFile writes a shorter title and an unquoted
// DATAPACKING, dnssetbl/combineFile.f90:59-61).
void put_header(std::string& out, int format, int style, double time, int nstep, int nproc, int nx, int nyz, int nz) {
    char buf[256];
    if (format == TBL_TP_DNSSETBL && style == 1)
        snprintf(buf, sizeof buf, "TITLE =\"%20.10f%9d%3d\"\n", time, nstep, nproc);
    else
        snprintf(buf, sizeof buf, "TITLE =\"%20.10f%9d\"\n", time, nstep);
    out += buf;
    if (format == TBL_TP_DNSTBL2)
        out += " Variables = \"x\",\"y\",\"z\",\"U\",\"V\",\"W\",\"P\",\"Um\",\"Vm\",\"Wm\",\"Uf\",\"Vf\",\"Wf\",\"Wt\",\"Nk\"\n";
    else if (format == TBL_TP_ORIGINAL)
        out += " Variables = \"x\",\"y\",\"z\",\"U\",\"V\",\"W\",\"T\",\"P\"\n";
    else
        out += "Variables = \"x\",\"y\",\"z\",\"U\",\"V\",\"W\",\"P\"\n";
    if (format == TBL_TP_DNSSETBL && style == 2)
        snprintf(buf, sizeof buf, "ZONE k=%4d,j=%4d,i=%4d,DATAPACKING=POINT\n", nx, nyz, nz);
    else
        snprintf(buf, sizeof buf, "ZONE k=%4d,j=%4d,i=%4d,DATAPACKING=\"POINT\"\n", nx, nyz, nz);
    out += buf;
}

// One point record from the column values (x, y, z, then the data columns;
// for the 15-column format the last value is new(k)).
void put_row(std::string& out, int format, const double* c) {
    const int n = ncols(format);
    for (int q = 0; q < 3; ++q) put_f(out, c[q], 10, 6);
    const int ne = format == TBL_TP_DNSTBL2 ? 11 : n - 3;
    for (int q = 0; q < ne; ++q) put_e(out, c[3 + q]);
    if (format == TBL_TP_DNSTBL2) {
        char buf[32];
        snprintf(buf, sizeof buf, " %4d", (int)c[14]);
        out += buf;
    }
    out += "\n";
}

// Column values of point (i,j,k) (0-based) of a state.
void point_cols(int format, const tbl_mesh* m, const tbl_state* st, int nx, int ny, int i, int j, int k, double* c) {
    const size_t p = id3(nx, ny, i, j, k), q = (size_t)i + (size_t)nx * k;
    c[0] = m->x1[i]; c[1] = m->x2[j]; c[2] = m->x3[k];
    c[3] = st->u[p]; c[4] = st->v[p]; c[5] = st->w[p];
    if (format == TBL_TP_ORIGINAL) {
        c[6] = 0.0;  // T
        c[7] = st->p[p];
    } else {
        c[6] = st->p[p];
    }
    if (format == TBL_TP_DNSTBL2) {
        c[7] = st->usum2[q]; c[8] = st->vsum2[q]; c[9] = st->wsum2[q];
        c[10] = at3(st->uf, p); c[11] = at3(st->vf, p); c[12] = at3(st->wf, p);
        c[13] = st->wt[q];
        c[14] = (double)st->newk[k];
    }
}

bool write_file(const char* path, const std::string& s) {
    FILE* f = fopen(path, "wb");
    if (!f) return false;
    const bool ok = fwrite(s.data(), 1, s.size(), f) == s.size();
    return fclose(f) == 0 && ok;
}

// The monitor files are opened with ACCESS='APPEND' by the reference.
bool append_file(const char* path, const std::string& s) {
    FILE* f = fopen(path, "ab");
    if (!f) return false;
    const bool ok = fwrite(s.data(), 1, s.size(), f) == s.size();
    return fclose(f) == 0 && ok;
}

bool read_file(const char* path, std::string& s) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    char buf[1 << 16];
    size_t n;
    s.clear();
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
    fclose(f);
    return true;
}

// Splits off the first three records; returns the position after them.
bool header_lines(const std::string& s, std::string hdr[3], size_t& pos) {
    pos = 0;
    for (int q = 0; q < 3; ++q) {
        const size_t e = s.find('\n', pos);
        if (e == std::string::npos) return false;
        hdr[q] = s.substr(pos, e - pos);
        pos = e + 1;
    }
    return true;
}

// time and nstep from the title: 8X, F20.10, I9 (dnstbl2/dnstbl.f90:385 format 01)
bool parse_title(const std::string& t, double& time, int& nstep) {
    if (t.size() < 37) return false;
    time = strtod(t.substr(8, 20).c_str(), nullptr);
    nstep = (int)strtol(t.substr(28, 9).c_str(), nullptr, 10);
    return true;
}

// ZONE k=nx,j=ny,i=nz
bool parse_zone(const std::string& z, int& nx, int& ny, int& nz) {
    const char* s = z.c_str();
    const char *a = strstr(s, "k="), *b = strstr(s, "j="), *c = strstr(s, "i=");
    if (!a || !b || !c) return false;
    nx = atoi(a + 2); ny = atoi(b + 2); nz = atoi(c + 2);
    return nx > 0 && ny > 0 && nz > 0;
}

// Whitespace-separated numbers from pos on; Ew.d values with a three-digit
// exponent and no E ("0.1+100") are read too.
bool parse_numbers(const std::string& s, size_t pos, size_t count, std::vector<double>& out) {
    out.clear();
    out.reserve(count);
    const char* p = s.c_str() + pos;
    const char* end = s.c_str() + s.size();
    std::string tok;
    while (out.size() < count) {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
        if (p >= end) return false;
        const char* q = p;
        while (q < end && !(*q == ' ' || *q == '\n' || *q == '\r' || *q == '\t')) ++q;
        tok.assign(p, q);
        for (size_t k = 1; k < tok.size(); ++k)
            if ((tok[k] == '+' || tok[k] == '-') && isdigit((unsigned char)tok[k - 1])) {
                tok.insert(k, 1, 'E');
                break;
            }
        char* e = nullptr;
        errno = 0;
        const double v = strtod(tok.c_str(), &e);
        if (e == tok.c_str()) return false;
        out.push_back(v);
        p = q;
    }
    return true;
}

// One Fortran Ew.d input field (list of characters already cut to the field
// width), read as a formatted READ does with the default BLANK='NULL':
// blanks are ignored, an all-blank field is zero, the exponent may be written
// with E, D or Q, or as a bare sign ("0.5+02"), and a mantissa without a
// decimal point carries d implied decimal places.  False when the field is
// not a number.
bool parse_fortran_e(const std::string& field, int d, double& v) {
    std::string t;
    for (char ch : field)
        if (ch != ' ' && ch != '\t' && ch != '\r' && ch != '\n') t += ch;
    if (t.empty()) {
        v = 0.0;
        return true;
    }
    size_t p = 0;
    std::string mant;
    if (t[p] == '+' || t[p] == '-') mant += t[p++];
    bool digits = false, point = false;
    for (; p < t.size(); ++p) {
        const char ch = t[p];
        if (isdigit((unsigned char)ch)) { mant += ch; digits = true; }
        else if (ch == '.' && !point) { mant += ch; point = true; }
        else break;
    }
    if (!digits) return false;
    long ex = 0;
    if (p < t.size()) {
        char ch = (char)toupper((unsigned char)t[p]);
        if (ch == 'E' || ch == 'D' || ch == 'Q') ch = t[++p];
        if (p >= t.size()) return false;
        size_t q = p;
        if (ch == '+' || ch == '-') ++q;
        if (q >= t.size()) return false;
        for (size_t r = q; r < t.size(); ++r)
            if (!isdigit((unsigned char)t[r])) return false;
        ex = strtol(t.c_str() + p, nullptr, 10);
    }
    if (!point) ex -= d;
    char buf[96];
    snprintf(buf, sizeof buf, "%sE%ld", mant.c_str(), ex);
    errno = 0;
    char* e = nullptr;
    v = strtod(buf, &e);
    return e != buf && *e == 0;
}

// 0-based k range of rank r's restart file.  dnstbl2/originalTBL: istart..iend
// of the (nz-1)/P partition from k = 2, with the wall plane on rank 0 and the
// top plane on the last rank (:469-485); dnssetbl: b(id)..e(id) of its nz/P
// partition (dnssetbl.f90:78-92, :922).
void rank_range(int format, int nz, int P, int r, int& k0, int& k1) {
    if (format == TBL_TP_DNSSETBL) {
        int it1 = nz / P, b = 0;
        const int it2 = P - nz % P;
        for (int q = 0; q <= r; ++q) {
            if (q == it2) it1 = it1 + 1;
            k0 = b;
            k1 = b + it1 - 1;
            b = k1 + 1;
        }
        return;
    }
    const int loc = (nz - 1) / P;
    const int bn = 1 + r * loc;
    const int en = r < P - 1 ? bn + loc - 1 : nz - 2;
    k0 = r == 0 ? bn - 1 : bn;
    k1 = r == P - 1 ? en + 1 : en;
}

std::string rank_path(const char* dir, int format, int r) {
    char name[64];
    snprintf(name, sizeof name, format == TBL_TP_DNSSETBL ? "/3D%03d.dat" : "/3D%03d.tp", r + 1);
    return std::string(dir) + name;
}

int write_range(const char* path, int format, const tbl_mesh* m, const tbl_state* st, int nx, int ny, int nz,
                int j0, int j1, int k0, int k1, int style, int nproc) {
    std::string out;
    out.reserve((size_t)nx * (j1 - j0 + 1) * (k1 - k0 + 1) * (34 + 23 * 12) + 1024);
    if (style) put_header(out, format, style, st->time, st->nstep, nproc, nx, j1 - j0 + 1, nz);
    double c[15];
    for (int i = 0; i < nx; ++i) {
        out += "\n";
        for (int j = j0; j <= j1; ++j) {
            out += "\n";
            for (int k = k0; k <= k1; ++k) {
                point_cols(format, m, st, nx, ny, i, j, k, c);
                put_row(out, format, c);
            }
        }
    }
    return write_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

bool state_ok(int format, const tbl_state* st) {
    if (!st || !st->u || !st->v || !st->w || !st->p) return false;
    if (format == TBL_TP_DNSTBL2 && (!st->usum2 || !st->vsum2 || !st->wsum2 || !st->wt || !st->newk)) return false;
    return true;
}

bool mesh_ok(const tbl_mesh* m) { return m && m->x1 && m->x2 && m->x3; }

}  // namespace

extern "C" {

int tbl_tp_write(const char* path, int32_t format, const tbl_mesh* mesh, const tbl_state* st, int32_t nx,
                 int32_t ny, int32_t nz, int32_t j0, int32_t j1, int32_t k0, int32_t k1, int32_t header,
                 int32_t nproc) {
    if (!path || !valid_format(format) || !mesh_ok(mesh) || !state_ok(format, st)) return TBL_ERR_BAD_ARG;
    if (nx < 1 || ny < 1 || nz < 1 || j0 < 1 || j1 > ny || j0 > j1 || k0 < 1 || k1 > nz || k0 > k1) return TBL_ERR_BAD_ARG;
    if (header < 0 || header > 2) return TBL_ERR_BAD_ARG;
    return write_range(path, format, mesh, st, nx, ny, nz, j0 - 1, j1 - 1, k0 - 1, k1 - 1, header, nproc);
}

int tbl_tp_write_ranks(const char* dir, int32_t format, const tbl_mesh* mesh, const tbl_state* st, int32_t nx,
                       int32_t ny, int32_t nz, int32_t nproc) {
    if (!dir || !valid_format(format) || !mesh_ok(mesh) || !state_ok(format, st)) return TBL_ERR_BAD_ARG;
    if (nx < 1 || ny < 3 || nz < 3 || nproc < 1 || nproc > 999) return TBL_ERR_BAD_ARG;
    for (int r = 0; r < nproc; ++r) {
        int k0, k1;
        rank_range(format, nz, nproc, r, k0, k1);
        if (k1 < k0) return TBL_ERR_BAD_ARG;
        const int s = write_range(rank_path(dir, format, r).c_str(), format, mesh, st, nx, ny, nz, 1, ny - 2, k0, k1,
                                  r == 0 ? 1 : 0, nproc);
        if (s != TBL_OK) return s;
    }
    return TBL_OK;
}

int tbl_tp_merge(const char* dir, int32_t format, int32_t nz, int32_t nproc, const char* out_path) {
    if (!dir || !out_path || !valid_format(format) || nz < 3 || nproc < 1 || nproc > 999) return TBL_ERR_BAD_ARG;
    const int nc = ncols(format);
    std::string s, hdr[3];
    size_t pos;
    if (!read_file(rank_path(dir, format, 0).c_str(), s)) return TBL_ERR_IO;
    if (!header_lines(s, hdr, pos)) return TBL_ERR_IO;
    double time;
    int nstep, nx, nyi, nzh;
    if (!parse_title(hdr[0], time, nstep) || !parse_zone(hdr[2], nx, nyi, nzh)) return TBL_ERR_IO;
    const int ny = nyi + 2;
    std::vector<double> data((size_t)nx * ny * nz * nc, 0.0), vals;
    auto D = [&](int i, int j, int k, int q) -> double& { return data[id3(nx, ny, i, j, k) * nc + q]; };
    for (int r = 0; r < nproc; ++r) {
        int k0, k1;
        rank_range(format, nz, nproc, r, k0, k1);
        if (r > 0) {
            if (!read_file(rank_path(dir, format, r).c_str(), s)) return TBL_ERR_IO;
            pos = 0;
        }
        const size_t cnt = (size_t)nx * nyi * (k1 - k0 + 1) * nc;
        if (!parse_numbers(s, pos, cnt, vals)) return TBL_ERR_IO;
        size_t t = 0;
        for (int i = 0; i < nx; ++i)
            for (int j = 1; j <= ny - 2; ++j)
                for (int k = k0; k <= k1; ++k)
                    for (int q = 0; q < nc; ++q) D(i, j, k, q) = vals[t++];
    }
    // Ghost rows: the velocities (and dnssetbl's pressure, which its merger
    // holds as Ut(:,:,:,4)) periodic, Ut(:,1,:,:) = Ut(:,ny-1,:,:) and
    // Ut(:,ny,:,:) = Ut(:,2,:,:); the (i,k) columns as on every row; the
    // remaining columns, which the mergers leave unset, zero.  x2(1) = 0 and
    // x2(ny) continues the uniform spacing (the mergers write the literal
    // span 4.0 of the reference's own domain).
    int periodic[4] = {3, 4, 5, format == TBL_TP_DNSSETBL ? 6 : (format == TBL_TP_ORIGINAL ? 6 : -1)};
    const double dy = D(0, 2, 0, 1) - D(0, 1, 0, 1);
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) {
            for (int a = 0; a < 4; ++a) {
                const int q = periodic[a];
                if (q < 0) continue;
                D(i, 0, k, q) = D(i, ny - 2, k, q);
                D(i, ny - 1, k, q) = D(i, 1, k, q);
            }
            const int same[] = {0, 2, 7, 8, 9, 13, 14};
            for (int q : same) {
                if (q >= nc || (format != TBL_TP_DNSTBL2 && q > 2)) continue;
                D(i, 0, k, q) = D(i, 1, k, q);
                D(i, ny - 1, k, q) = D(i, 1, k, q);
            }
            D(i, 0, k, 1) = 0.0;
            D(i, ny - 1, k, 1) = D(0, 1, 0, 1) + (ny - 2) * dy;
        }
    std::string out;
    out.reserve((size_t)nx * ny * nz * (34 + 23 * (nc - 3)) + 1024);
    put_header(out, format, 2, time, nstep, nproc, nx, ny, nz);
    for (int i = 0; i < nx; ++i) {
        out += "\n";
        for (int j = 0; j < ny; ++j) {
            out += "\n";
            for (int k = 0; k < nz; ++k) put_row(out, format, &D(i, j, k, 0));
        }
    }
    return write_file(out_path, out) ? TBL_OK : TBL_ERR_IO;
}

int tbl_tp_read(const char* path, int32_t format, int32_t nx, int32_t ny, int32_t nz, double* x1, double* x2,
                double* x3, tbl_state* st) {
    if (!path || !valid_format(format) || !st || nx < 1 || ny < 1 || nz < 1) return TBL_ERR_BAD_ARG;
    std::string s, hdr[3];
    size_t pos;
    if (!read_file(path, s)) return TBL_ERR_IO;
    if (!header_lines(s, hdr, pos)) return TBL_ERR_IO;
    double time;
    int nstep, znx, zny, znz;
    if (!parse_title(hdr[0], time, nstep) || !parse_zone(hdr[2], znx, zny, znz)) return TBL_ERR_IO;
    if (znx != nx || zny != ny || znz != nz) return TBL_ERR_BAD_ARG;
    const int nc = ncols(format);
    std::vector<double> vals;
    if (!parse_numbers(s, pos, (size_t)nx * ny * nz * nc, vals)) return TBL_ERR_IO;
    const int ip = format == TBL_TP_ORIGINAL ? 7 : 6;
    size_t t = 0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k, t += nc) {
                const double* c = &vals[t];
                const size_t p = id3(nx, ny, i, j, k), q = (size_t)i + (size_t)nx * k;
                if (x1 && j == 0 && k == 0) x1[i] = c[0];
                if (x2 && i == 0 && k == 0) x2[j] = c[1];
                if (x3 && i == 0 && j == 0) x3[k] = c[2];
                if (st->u) st->u[p] = c[3];
                if (st->v) st->v[p] = c[4];
                if (st->w) st->w[p] = c[5];
                if (st->p) st->p[p] = c[ip];
                if (format != TBL_TP_DNSTBL2) continue;
                // the (i,k) columns repeat on every row; the last one read stays, as in the reference's read loop
                if (st->usum2) st->usum2[q] = c[7];
                if (st->vsum2) st->vsum2[q] = c[8];
                if (st->wsum2) st->wsum2[q] = c[9];
                if (st->uf) st->uf[p] = c[10];
                if (st->vf) st->vf[p] = c[11];
                if (st->wf) st->wf[p] = c[12];
                if (st->wt) st->wt[q] = c[13];
                if (st->newk) st->newk[k] = (int32_t)c[14];
            }
    st->time = time;
    st->nstep = nstep;
    return TBL_OK;
}

int tbl_counters_write(const char* dir, int32_t nz, int32_t cnt, int32_t nproc, int32_t cnt2) {
    if (!dir) return TBL_ERR_BAD_ARG;
    char buf[128];
    snprintf(buf, sizeof buf, "%12d%12d%12d\n", nz, cnt, nproc);
    if (!write_file((std::string(dir) + "/cnt").c_str(), buf)) return TBL_ERR_IO;
    snprintf(buf, sizeof buf, "%12d\n", cnt2);
    if (!write_file((std::string(dir) + "/cnt2").c_str(), buf)) return TBL_ERR_IO;
    return TBL_OK;
}

int tbl_counters_read(const char* dir, int32_t* nz, int32_t* cnt, int32_t* nproc, int32_t* cnt2) {
    if (!dir || !nz || !cnt || !nproc || !cnt2) return TBL_ERR_BAD_ARG;
    std::string s;
    std::vector<double> v;
    if (!read_file((std::string(dir) + "/cnt").c_str(), s) || !parse_numbers(s, 0, 3, v)) return TBL_ERR_IO;
    *nz = (int32_t)v[0]; *cnt = (int32_t)v[1]; *nproc = (int32_t)v[2];
    if (!read_file((std::string(dir) + "/cnt2").c_str(), s) || !parse_numbers(s, 0, 1, v)) return TBL_ERR_IO;
    *cnt2 = (int32_t)v[0];
    return TBL_OK;
}

// dnssetbl's Input/statData.dat: per k, usum2(irec,k), vsum2(irec,k),
// wsum2(irec,k), Wt(1,k) and new(k), FORMAT(4(1X,F15.7),I5.3)
// (dnssetbl.f90:1203-1208, read at :136-140).  Seven decimals: a restart
// through this file rounds the recycling means and the blend weights.
int tbl_statdata_write(const char* path, int32_t nx, int32_t nz, int32_t irec, const tbl_state* st) {
    if (!path || !st || !st->usum2 || !st->vsum2 || !st->wsum2 || !st->wt || !st->newk) return TBL_ERR_BAD_ARG;
    if (nx < 1 || nz < 1 || irec < 1 || irec > nx) return TBL_ERR_BAD_ARG;
    std::string out;
    char buf[160];
    for (int k = 0; k < nz; ++k) {
        const size_t q = (size_t)(irec - 1) + (size_t)nx * k;
        snprintf(buf, sizeof buf, " %15.7f %15.7f %15.7f %15.7f%5.3d\n", st->usum2[q], st->vsum2[q], st->wsum2[q],
                 st->wt[(size_t)nx * k], st->newk[k]);
        out += buf;
    }
    return write_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

int tbl_statdata_read(const char* path, int32_t nx, int32_t nz, int32_t irec, tbl_state* st) {
    if (!path || !st || !st->usum2 || !st->vsum2 || !st->wsum2 || !st->wt || !st->newk) return TBL_ERR_BAD_ARG;
    if (nx < 1 || nz < 1 || irec < 1 || irec > nx) return TBL_ERR_BAD_ARG;
    std::string s;
    std::vector<double> v;
    if (!read_file(path, s) || !parse_numbers(s, 0, (size_t)5 * nz, v)) return TBL_ERR_IO;
    for (int k = 0; k < nz; ++k) {
        const size_t q = (size_t)(irec - 1) + (size_t)nx * k;
        st->usum2[q] = v[5 * k]; st->vsum2[q] = v[5 * k + 1]; st->wsum2[q] = v[5 * k + 2];
        st->wt[(size_t)nx * k] = v[5 * k + 3];
        st->newk[k] = (int32_t)v[5 * k + 4];
    }
    return TBL_OK;
}

// The inflow mean profile: 37 records read with FORMAT(24X,E18.8), the value
// of record 37 kept for every plane above it (dnstbl2/dnstbl.f90:322-345;
// the same format in originalTBL/fnldnstbl.f90:411-423 and dnssetbl's
// Input/initProf.dat, dnssetbl/dnssetbl.f90:105-114).  A record shorter than
// 42 characters is padded with blanks, as a formatted READ pads it.
int tbl_inflow_profile_read(const char* path, int32_t nz, double* ume1) {
    if (!path || !ume1 || nz < 1) return TBL_ERR_BAD_ARG;
    std::string s;
    if (!read_file(path, s)) return TBL_ERR_IO;
    double last = 0.0;
    size_t pos = 0;
    for (int k = 0; k < TBL_INFLOW_RECORDS; ++k) {
        if (pos >= s.size()) return TBL_ERR_IO;  // fewer than 37 records
        size_t e = s.find('\n', pos);
        if (e == std::string::npos) e = s.size();
        std::string rec = s.substr(pos, e - pos);
        pos = e + 1;
        if (rec.size() < 42) rec.resize(42, ' ');
        double v = 0.0;
        if (!parse_fortran_e(rec.substr(24, 18), 8, v)) return TBL_ERR_IO;
        if (k < nz) ume1[k] = v;
        last = v;
    }
    for (int k = TBL_INFLOW_RECORDS; k < nz; ++k) ume1[k] = last;
    return TBL_OK;
}

// The same file from a profile: per record "(1X,I4,1X,E18.8,1X,E18.8)" =
// k, x3(k) in the 24 skipped columns, then Ume1(k) in E18.8 (9 significant
// digits) -- the 37 records the reference reads.  Planes above 37 are not
// written (the reader repeats record 37 there).
int tbl_inflow_profile_write(const char* path, int32_t nz, const double* x3, const double* ume1) {
    if (!path || !x3 || !ume1 || nz < TBL_INFLOW_RECORDS) return TBL_ERR_BAD_ARG;
    std::string out;
    for (int k = 0; k < TBL_INFLOW_RECORDS; ++k) {
        char buf[32];
        snprintf(buf, sizeof buf, " %4d", k + 1);
        out += buf;
        std::string a, b;
        put_e_wd(a, x3[k], 18, 8);
        put_e_wd(b, ume1[k], 18, 8);
        out += a;   // " " + 18 columns: 24 columns in all before the value
        out += b.substr(1);
        out += "\n";
    }
    return write_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// ------------------------------------------------------------ monitor files
// The files the reference's rank 0 writes during a run, record for record.
// Those it opens with ACCESS='APPEND' get the records appended; the others
// are rewritten.  (nx,nz) arrays are in Fortran order, i fastest.

// massflow.xy: time and the five plane mass fluxes UbDNS, FORMAT(6(1X,F15.7))
// (dnstbl2/dnstbl.f90:1613-1615, :2390).
int tbl_monitor_massflow(const char* path, double time, const double* ubulk) {
    if (!path || !ubulk) return TBL_ERR_BAD_ARG;
    std::string out;
    put_fw(out, time, 1, 15, 7);
    for (int q = 0; q < 5; ++q) put_fw(out, ubulk[q], 1, 15, 7);
    out += "\n";
    return append_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// numrcltauwall.xy after a 500-step wall-shear window: per i = 2..nx-1 the
// time, x1(i), the span-mean shear sumxz(i)/(ny-2) and Cf =
// 2 (sumxz(i)/(Ue Ue (ny-2))), FORMAT(4(1X,F15.7)) (:1674-1679, :2392);
// tauw_window is sumxz already divided by 500 (:1670).
int tbl_monitor_tauwall(const char* path, double time, int32_t nx, int32_t ny, double ue, const double* x1,
                        const double* tauw_window) {
    if (!path || !x1 || !tauw_window || nx < 3 || ny < 3) return TBL_ERR_BAD_ARG;
    std::string out;
    const double span = (double)(ny - 2);
    for (int i = 1; i < nx - 1; ++i) {
        put_fw(out, time, 1, 15, 7);
        put_fw(out, x1[i], 1, 15, 7);
        put_fw(out, tauw_window[i] / span, 1, 15, 7);
        put_fw(out, 2.0 * (tauw_window[i] / (ue * ue * span)), 1, 15, 7);
        out += "\n";
    }
    return append_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// kineticenergy.dat: time and the fluctuation energy, FORMAT(2(2X,E20.10))
// (:1718-1721).
int tbl_monitor_kinetic_energy(const char* path, double time, double ke) {
    if (!path) return TBL_ERR_BAD_ARG;
    std::string out;
    put_ew(out, time, 2, 20, 10);
    put_ew(out, ke, 2, 20, 10);
    out += "\n";
    return append_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// lamda.dat after a rescaling: time, lamda, lamda03, FORMAT(3(2X,F20.10))
// (:2170-2174).
int tbl_monitor_lamda(const char* path, double time, double lamda, double lamda03) {
    if (!path) return TBL_ERR_BAD_ARG;
    std::string out;
    put_fw(out, time, 2, 20, 10);
    put_fw(out, lamda, 2, 20, 10);
    put_fw(out, lamda03, 2, 20, 10);
    out += "\n";
    return append_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// W.dat (rewritten): per i, per k: x1(i), x3(k), Wt(i,k), FORMAT(3(1X,F15.7))
// (:2180-2188, :2388).
int tbl_monitor_blend(const char* path, int32_t nx, int32_t nz, const double* x1, const double* x3, const double* wt) {
    if (!path || !x1 || !x3 || !wt || nx < 1 || nz < 1) return TBL_ERR_BAD_ARG;
    std::string out;
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) {
            put_fw(out, x1[i], 1, 15, 7);
            put_fw(out, x3[k], 1, 15, 7);
            put_fw(out, wt[(size_t)i + (size_t)nx * k], 1, 15, 7);
            out += "\n";
        }
    return write_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// boundarylthickness.dat (rewritten): per i: time, x1, bltkns, deltastar,
// theta, Ht, Reth, FORMAT(7(2X,F20.10)) (:2258-2267).
int tbl_monitor_bl_thickness(const char* path, double time, int32_t nx, const double* x1, const double* bltkns,
                             const double* deltastar, const double* theta, const double* ht, const double* reth) {
    if (!path || !x1 || !bltkns || !deltastar || !theta || !ht || !reth || nx < 1) return TBL_ERR_BAD_ARG;
    std::string out;
    for (int i = 0; i < nx; ++i) {
        const double c[7] = {time, x1[i], bltkns[i], deltastar[i], theta[i], ht[i], reth[i]};
        for (double v : c) put_fw(out, v, 2, 20, 10);
        out += "\n";
    }
    return write_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// k.dat (every 100th step of a rescaling): per k: k, new(k), eta(k),
// FORMAT(I5,2(F20.10)) (:2286-2292); new(k) is a REAL array there.
int tbl_monitor_knew(const char* path, int32_t nz, const int32_t* newk, const double* eta) {
    if (!path || !newk || !eta || nz < 1) return TBL_ERR_BAD_ARG;
    std::string out;
    char buf[32];
    for (int k = 0; k < nz; ++k) {
        snprintf(buf, sizeof buf, "%5d", k + 1);
        out += strlen(buf) > 5 ? std::string(5, '*') : std::string(buf);
        put_fw(out, (double)newk[k], 0, 20, 10);
        put_fw(out, eta[k], 0, 20, 10);
        out += "\n";
    }
    return append_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// meanvalues.dat (every 100th step of a rescaling): per i, per k: x1(i),
// x3(k), usum2, vsum2, wsum2, FORMAT(5(1X,F15.7)) (:2296-2302, :2387).
int tbl_monitor_meanvalues(const char* path, int32_t nx, int32_t nz, const double* x1, const double* x3,
                           const double* usum2, const double* vsum2, const double* wsum2) {
    if (!path || !x1 || !x3 || !usum2 || !vsum2 || !wsum2 || nx < 1 || nz < 1) return TBL_ERR_BAD_ARG;
    std::string out;
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) {
            const size_t q = (size_t)i + (size_t)nx * k;
            const double c[5] = {x1[i], x3[k], usum2[q], vsum2[q], wsum2[q]};
            for (double v : c) put_fw(out, v, 1, 15, 7);
            out += "\n";
        }
    return append_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// Umeanvalues.dat (rewritten at every rescaling): the same columns and
// x3(k)*Re, FORMAT(6(1X,F15.7)) (:2098-2104, :2386).
int tbl_monitor_umeanvalues(const char* path, int32_t nx, int32_t nz, const double* x1, const double* x3,
                            const double* usum2, const double* vsum2, const double* wsum2, double re) {
    if (!path || !x1 || !x3 || !usum2 || !vsum2 || !wsum2 || nx < 1 || nz < 1) return TBL_ERR_BAD_ARG;
    std::string out;
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) {
            const size_t q = (size_t)i + (size_t)nx * k;
            const double c[6] = {x1[i], x3[k], usum2[q], vsum2[q], wsum2[q], x3[k] * re};
            for (double v : c) put_fw(out, v, 1, 15, 7);
            out += "\n";
        }
    return write_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

// means, medians, taustress (rewritten at every rescaling): ONE record of
// four FORMAT(4(1X,F15.7)) fields per (i,k), i outer -- the averaged sums a,
// b, c and the temperature's, written as zero (no temperature here) --
// written with ADVANCE='NO' and closed by an empty list-directed WRITE
// (:2021-2049, :2385).
int tbl_monitor_averages(const char* path, int32_t nx, int32_t nz, const double* a, const double* b,
                         const double* c) {
    if (!path || !a || !b || !c || nx < 1 || nz < 1) return TBL_ERR_BAD_ARG;
    std::string out;
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) {
            const size_t q = (size_t)i + (size_t)nx * k;
            put_fw(out, a[q], 1, 15, 7);
            put_fw(out, b[q], 1, 15, 7);
            put_fw(out, c[q], 1, 15, 7);
            put_fw(out, 0.0, 1, 15, 7);
        }
    out += "\n";
    return write_file(path, out) ? TBL_OK : TBL_ERR_IO;
}

}  // extern "C"
