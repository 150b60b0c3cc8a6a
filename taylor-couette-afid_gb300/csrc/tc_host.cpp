// tc_host.cpp -- host-only parts of the library: bou.in reader, grid and
// coefficient construction, configuration checks.
//
// tc_read_bou follows ReadInputFile.F90:17-39: a header record (read with
// format a4 and discarded) precedes each list-directed value record.  As in
// Fortran list-directed input, values may be separated by blanks or commas,
// a record with too few values continues on the next record, `r*v` repeats
// a value, `/` ends the list leaving the remaining items unchanged, and the
// rest of the last record read is skipped.

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "tc_grid.h"

namespace tcgb {

namespace {

struct Item { bool is_int; void* p; };

// One list-directed READ starting at record `line`; advances `line`.
bool list_read(const std::vector<std::string>& recs, size_t& line, std::vector<Item> items,
               std::string& err) {
    size_t it = 0;
    while (it < items.size()) {
        if (line >= recs.size()) { err = "unexpected end of file"; return false; }
        std::string s = recs[line++];
        for (auto& c : s) if (c == ',' || c == '\t') c = ' ';
        std::istringstream in(s);
        std::string tok;
        bool slash = false;
        while (it < items.size() && in >> tok) {
            if (tok[0] == '/') { slash = true; break; }
            int rep = 1;
            size_t star = tok.find('*');
            if (star != std::string::npos) {
                rep = std::atoi(tok.substr(0, star).c_str());
                tok = tok.substr(star + 1);
                if (rep < 1) { err = "bad repeat count"; return false; }
            }
            size_t sl = tok.find('/');
            if (sl != std::string::npos) { tok = tok.substr(0, sl); slash = true; }
            for (int r = 0; r < rep && it < items.size(); ++r, ++it) {
                if (tok.empty()) continue;  // null value: item unchanged
                if (items[it].is_int) {
                    char* end = nullptr;
                    long v = std::strtol(tok.c_str(), &end, 10);
                    if (*end != '\0') { err = "integer expected, got '" + tok + "'"; return false; }
                    *(int*)items[it].p = (int)v;
                } else {
                    std::string t = tok;
                    for (auto& c : t) if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
                    char* end = nullptr;
                    double v = std::strtod(t.c_str(), &end);
                    if (*end != '\0' || t.empty()) { err = "real expected, got '" + tok + "'"; return false; }
                    *(double*)items[it].p = v;
                }
            }
            if (slash) break;
        }
        if (slash) return true;
    }
    return true;
}

inline double sq(double x) { return x * x; }

// The FFT engine's radices: every prime factor of a transform length must
// be one of these.
bool fft_length_ok(int n) {
    if (n < 1) return false;
    for (int p : {2, 3, 5, 7, 11, 13}) while (n % p == 0) n /= p;
    return n == 1;
}

}  // namespace

std::string validate(const tc_bou& b) {
    char buf[256];
    if (b.nrm < 3) return "NRM must be at least 3";
    if (b.nthm < 4 || b.nthm % 2) return "NTM must be even and at least 4";
    if (b.nzm < 2 || b.nzm % 2) return "NZM must be even and at least 2";
    if (!fft_length_ok(b.nthm / 2) || !fft_length_ok(b.nzm)) {
        std::snprintf(buf, sizeof buf, "NTM/2=%d and NZM=%d must have no prime factor above 13", b.nthm / 2, b.nzm);
        return buf;
    }
    if (b.nthm > 4096 || b.nzm > 1536 || b.nrm > 4096)
        return "grid exceeds the supported maximum (NTM <= 4096, NZM <= 1536, NRM <= 4096)";
    if (b.nsst < 1 || b.nsst > 3) return "NSST must be 1 (AB2) or 3 (RK3)";
    if (b.istr != 0 && b.istr != 4 && b.istr != 6)
        return "ISTR must be 0, 4 or 6 (the grids CreateGrid.F90 defines)";
    if (b.istr == 6 && (int)b.str < 0) return "ISTR=6 needs STR3 >= 0";
    if (!(b.rext > b.rint) || !(b.rint > 0.0)) return "need 0 < RINT < REXT";
    if (!(b.ren > 0.0)) return "1/NU must be positive";
    if (!(b.alx3 > 0.0) || !(b.lamb > 0.0)) return "ALX3D and LAMB must be positive";
    int ntott = b.minstrt * b.multmin, ntotz = b.minstrz * b.multmin;
    if (ntott + ntotz != 0 && (ntott == 0 || ntotz == 0))
        return "patterned slip needs MINSTRT*MULTMIN and MINSTRZ*MULTMIN both non-zero "
               "(SlipBCs.F90:58-59 divides by each)";
    long long cells = (long long)b.nthm * b.nzm * b.nrm;
    if (cells > (1LL << 31) - 1) return "more than 2^31-1 cells";
    return "";
}

void time_march_scheme(int nsst, double gam[3], double rom[3], double alm[3]) {
    if (nsst > 1) {
        gam[0] = 8.0 / 15.0; gam[1] = 5.0 / 12.0; gam[2] = 3.0 / 4.0;
        rom[0] = 0.0; rom[1] = -17.0 / 60.0; rom[2] = -5.0 / 12.0;
    } else {
        gam[0] = 1.5; gam[1] = 0.0; gam[2] = 0.0;
        rom[0] = -0.5; rom[1] = 0.0; rom[2] = 0.0;
    }
    for (int i = 0; i < 3; ++i) alm[i] = gam[i] + rom[i];
}

std::string build_grid(const tc_bou& b, Grid& g) {
    std::string v = validate(b);
    if (!v.empty()) return v;
    const int nthm = b.nthm, nzm = b.nzm, nrm = b.nrm, nr = nrm + 1;
    g.nthm = nthm; g.nzm = nzm; g.nrm = nrm; g.nr = nr;
    for (auto* a : {&g.rc, &g.rm, &g.g2rc, &g.g2rm, &g.usrc, &g.usrm, &g.udx1vis1, &g.udx1vis2,
                    &g.udx1qm, &g.udx2c, &g.udx2m, &g.rudx2c, &g.udx2rm, &g.pvol, &g.udx2mm, &g.udx2cc,
                    &g.ap1j, &g.am1j,
                    &g.ac1j, &g.ap2j, &g.am2j, &g.ac2j, &g.ap2je, &g.am2je, &g.ac2je, &g.ap3j,
                    &g.am3j, &g.ac3j, &g.apph, &g.amph, &g.acph})
        a->assign(nr, 0.0);
    // Reference arrays are 1-based; R(a, k) addresses a(k).
    auto R = [](std::vector<double>& a, int k) -> double& { return a[k - 1]; };

    g.pi = 2.0 * std::asin(1.0);                                  // CreateGrid.F90:24
    g.dxt = ((double)nthm * b.lamb) / (2.0 * g.pi);               // CreateGrid.F90:28-34
    g.dxz = (double)nzm / b.alx3;
    g.dxr = (double)nrm / 1.0;
    g.dxtq = g.dxt * g.dxt; g.dxzq = g.dxz * g.dxz; g.dxrq = g.dxr * g.dxr;
    const double dxr = g.dxr, dxrq = g.dxrq;

    auto& rc = g.rc;
    if (b.istr == 0) {                                            // CreateGrid.F90:85-90
        for (int k = 1; k <= nr; ++k) R(rc, k) = (b.rext - b.rint) * ((double)(k - 1) / (double)nrm) + b.rint;
    } else if (b.istr == 4) {                                     // CreateGrid.F90:99-105
        double tstr = std::tanh(b.str);
        R(rc, 1) = b.rint;
        for (int k = 2; k <= nr; ++k) {
            double z2dp = (double)(2 * k - nr - 1) / (double)nrm;
            R(rc, k) = (1.0 + std::tanh(b.str * z2dp) / tstr) * 0.5 * (b.rext - b.rint) + b.rint;
        }
    } else {                                                      // CreateGrid.F90:109-128
        int nclip = (int)b.str, nrmo = nr + 2 * nclip;
        std::vector<double> etaz(nr + 1);
        for (int k = 1; k <= nr; ++k)
            etaz[k] = std::cos(g.pi * ((double)(k + nclip) - 0.5) / (double)nrmo);
        double delet = etaz[1] - etaz[nr];
        for (int k = 1; k <= nr; ++k) etaz[k] = etaz[k] / (0.5 * delet);
        R(rc, 1) = b.rint;
        for (int k = 2; k <= nrm; ++k) R(rc, k) = (b.rext - b.rint) * (1.0 - etaz[k]) * 0.5 + b.rint;
        R(rc, nr) = b.rext;
    }
    for (int k = 1; k <= nrm; ++k) {                              // CreateGrid.F90:136-139
        R(g.rm, k) = (R(rc, k) + R(rc, k + 1)) * 0.5;
        R(g.g2rm, k) = (R(rc, k + 1) - R(rc, k)) * dxr;
    }
    R(g.g2rc, 1) = (R(rc, 2) - R(rc, 1)) * dxr;                   // CreateGrid.F90:141-151
    for (int k = 2; k <= nrm; ++k) R(g.g2rc, k) = (R(rc, k + 1) - R(rc, k - 1)) * dxr * 0.5;
    R(g.g2rc, nr) = (R(rc, nr) - R(rc, nrm)) * dxr;
    for (int k = 1; k <= nrm; ++k) {                              // CreateGrid.F90:156-166
        R(g.udx1vis1, k) = 2.0 * g.dxt / (sq(R(g.rm, k)) * b.ren);
        R(g.udx2rm, k) = dxr / (R(g.g2rm, k) * R(g.rm, k));
        R(g.udx2m, k) = dxr / R(g.g2rm, k);
        R(g.udx2c, k) = dxr / R(g.g2rc, k);
        R(g.rudx2c, k) = R(g.udx2c, k) * R(rc, k);
        R(g.usrm, k) = 1.0 / R(g.rm, k);
        R(g.udx1qm, k) = g.dxtq / sq(R(g.rm, k));
        R(g.pvol, k) = sq(R(rc, k + 1)) - sq(R(rc, k));
    }
    R(g.udx2c, nr) = dxr / R(g.g2rc, nr);                         // CreateGrid.F90:167
    {   // CreateGrid.F90:141-153,160,173: g2rmm and g2rcc (statistics only).  rm(nr) is never
        // set by CreateGrid and stays 0, so g2rmm(nrm) and udx2mm(nrm) use it.
        std::vector<double> g2rmm(nr, 0.0), g2rcc(nr, 0.0);
        R(g2rmm, 1) = (R(g.rm, 2) - R(g.rm, 1)) * dxr;
        R(g2rcc, 1) = (R(rc, 2) - R(rc, 1)) * dxr;
        for (int k = 2; k <= nrm; ++k) {
            R(g2rmm, k) = (R(g.rm, k + 1) - R(g.rm, k - 1)) * dxr;
            R(g2rcc, k) = (R(rc, k + 1) - R(rc, k - 1)) * dxr;
        }
        R(g2rmm, nr) = (R(g.rm, nr) - R(g.rm, nrm)) * dxr;
        R(g2rcc, nr) = (R(rc, nr) - R(rc, nrm)) * dxr;
        for (int k = 1; k <= nrm; ++k) R(g.udx2mm, k) = dxr / R(g2rmm, k);
        for (int k = 1; k <= nr; ++k) R(g.udx2cc, k) = dxr / R(g2rcc, k);
    }
    for (int k = 1; k <= nr; ++k) {                               // CreateGrid.F90:169-174
        R(g.udx1vis2, k) = g.dxt / (R(rc, k) * b.ren);
        R(g.usrc, k) = 1.0 / R(rc, k);
    }
    auto& rm = g.rm; auto& g2rm = g.g2rm; auto& g2rc = g.g2rc;
    // q1 (CreateGrid.F90:191-238)
    for (int kc = 2; kc <= nrm - 1; ++kc) {
        double a22 = dxrq / R(g2rm, kc) / R(rm, kc);
        double a22p = +a22 * R(rc, kc + 1) / R(g2rc, kc + 1);
        double a22m = +a22 * R(rc, kc) / R(g2rc, kc);
        R(g.ap1j, kc) = a22p; R(g.am1j, kc) = a22m;
        R(g.ac1j, kc) = -(a22p + a22m) - 1.0 / sq(R(rm, kc));
    }
    {
        int kc = nrm;
        double a22 = dxrq / (R(g2rm, kc) * R(rm, kc));
        double apjjc = a22 * R(rc, kc + 1) / R(g2rc, kc + 1);
        double amjjc = a22 * R(rc, kc) / R(g2rc, kc);
        R(g.ap1j, kc) = 2.0 * apjjc;
        R(g.ac1j, kc) = -2.0 * apjjc - amjjc - 1.0 / sq(R(rm, kc));
        R(g.am1j, kc) = amjjc;
        // The reference stores these in the inner (index 1) slot and the
        // inner-wall block below overwrites them; the outer slot stays 0.
    }
    {
        int kc = 1;
        double urpp = 1.0 / (R(g2rm, kc) * R(g2rc, kc + 1));
        double a22 = dxrq / R(g2rm, kc) / R(rm, kc);
        double a22p = +a22 * R(rc, kc + 1) / R(g2rc, kc + 1);
        double a22m = +a22 * R(rc, kc) / R(g2rc, kc);
        R(g.ap1j, kc) = a22p;
        R(g.am1j, kc) = 2.0 * a22m;
        R(g.ac1j, kc) = -(a22p + 2.0 * a22m) - 1.0 / sq(R(rm, kc));
        g.ap1j_fs[0] = std::pow(R(rc, kc + 1), 3) / (sq(R(rm, kc)) * R(rm, kc + 1)) * dxrq * urpp;
        g.ac1j_fs[0] = -std::pow(R(rc, kc + 1), 3) / std::pow(R(rm, kc), 3) * dxrq * urpp;
        g.am1j_fs[0] = 0.0;
        g.ap1j_fs[1] = g.ac1j_fs[1] = g.am1j_fs[1] = 0.0;
    }
    // q2 (CreateGrid.F90:241-276)
    R(g.ac2j, 1) = 1.0; R(g.ac2j, nr) = 1.0;
    for (int kc = 2; kc <= nrm; ++kc) {
        int km = kc - 1, kp = kc + 1;
        double a22 = R(rc, kc) * dxrq / R(g2rc, kc);
        double a22p = 1.0 / (R(rm, kc) * R(g2rm, kc));
        double a22m = 1.0 / (R(rm, km) * R(g2rm, km));
        R(g.ap2j, kc) = a22 * a22p; R(g.am2j, kc) = a22 * a22m;
        R(g.ac2j, kc) = -(a22 * a22p + a22 * a22m);
        double ugmm = dxrq / R(g2rc, kc);
        double e22p = R(rm, kc) / (R(rc, kp) * R(g2rm, kc));
        double e22m = R(rm, km) / (R(rc, km) * R(g2rm, km));
        double e22 = (R(rm, kc) / R(g2rm, kc) + R(rm, km) / R(g2rm, km)) / R(rc, kc);
        R(g.ap2je, kc) = e22p * ugmm; R(g.am2je, kc) = e22m * ugmm;
        R(g.ac2je, kc) = -e22 * ugmm - 1.0 / sq(R(rc, kc));
    }
    // q3 (CreateGrid.F90:279-322)
    for (int kc = 2; kc <= nrm - 1; ++kc) {
        double a22 = dxrq / R(g2rm, kc) / R(rm, kc);
        double a22p = +a22 * R(rc, kc + 1) / R(g2rc, kc + 1);
        double a22m = +a22 * R(rc, kc) / R(g2rc, kc);
        R(g.ap3j, kc) = a22p; R(g.am3j, kc) = a22m; R(g.ac3j, kc) = -(a22p + a22m);
    }
    {
        double a22 = dxrq / R(g2rm, 1) / R(rm, 1);
        double a22p = +a22 * R(rc, 2) / R(g2rc, 2);
        double a22m = +a22 * R(rc, 1) / R(g2rc, 1);
        R(g.am3j, 1) = 0.0; R(g.ap3j, 1) = a22p; R(g.ac3j, 1) = -(a22p + 2.0 * a22m);
        g.am3j_fs[0] = 0.0; g.ap3j_fs[0] = a22p; g.ac3j_fs[0] = -(a22p);
    }
    {
        int kc = nrm;
        double a22 = dxrq / R(g2rm, kc) / R(rm, kc);
        double a22m = +a22 * R(rc, kc) / R(g2rc, kc);
        double a22p = +a22 * R(rc, kc + 1) / R(g2rc, kc + 1);
        R(g.am3j, kc) = a22m; R(g.ap3j, kc) = 0.0; R(g.ac3j, kc) = -(a22m + 2.0 * a22p);
        g.am3j_fs[1] = a22m; g.ap3j_fs[1] = 0.0; g.ac3j_fs[1] = -(a22m);
    }
    // pressure operator (InitPressureSolver.F90:22-32); kmc(1) = kpc(nrm) = 0
    for (int kc = 1; kc <= nrm; ++kc) {
        int kmc = (kc == 1) ? 0 : 1, kpc = (kc == nrm) ? 0 : 1;
        int kp = kc + kpc;
        double a22icc = R(rc, kc) * kmc * dxrq / R(g2rc, kc);
        double a22icp = R(rc, kp) * kpc * dxrq / R(g2rc, kp);
        double ac2 = -(a22icc + a22icp);
        double ugmmm = 1.0 / (R(rm, kc) * R(g2rm, kc));
        R(g.amph, kc) = a22icc * ugmmm;
        R(g.apph, kc) = a22icp * ugmmm;
        R(g.acph, kc) = ac2 * ugmmm;
    }
    // modified wavenumbers (InitPressureSolver.F90:41-66), with the negative-frequency form above
    // nzm/2+1 and nthm/2+1
    g.ak3.assign(nzm, 0.0);
    for (int j = 1; j <= nzm; ++j) {
        double ao = (j <= nzm / 2 + 1) ? (j - 1) * 2.0 * g.pi : -(nzm - j + 1) * 2.0 * g.pi;
        g.ak3[j - 1] = 2.0 * (1.0 - std::cos(ao / nzm)) * sq((double)nzm / b.alx3);
    }
    g.ak1.assign(nthm, 0.0);
    for (int i = 1; i <= nthm; ++i) {
        double ap = (i <= nthm / 2 + 1) ? (i - 1) * 2.0 * g.pi : -(nthm - i + 1) * 2.0 * g.pi;
        g.ak1[i - 1] = 2.0 * (1.0 - std::cos(ap / nthm)) * g.dxtq;
    }
    return "";
}

const std::vector<double>* grid_array(const Grid& g, int which) {
    switch (which) {
        case TC_G_RC: return &g.rc;         case TC_G_RM: return &g.rm;
        case TC_G_G2RC: return &g.g2rc;     case TC_G_G2RM: return &g.g2rm;
        case TC_G_USRC: return &g.usrc;     case TC_G_USRM: return &g.usrm;
        case TC_G_UDX1VIS1: return &g.udx1vis1; case TC_G_UDX1VIS2: return &g.udx1vis2;
        case TC_G_UDX1QM: return &g.udx1qm; case TC_G_UDX2C: return &g.udx2c;
        case TC_G_UDX2M: return &g.udx2m;   case TC_G_RUDX2C: return &g.rudx2c;
        case TC_G_UDX2RM: return &g.udx2rm;
        case TC_G_AP1J: return &g.ap1j; case TC_G_AM1J: return &g.am1j; case TC_G_AC1J: return &g.ac1j;
        case TC_G_AP2J: return &g.ap2j; case TC_G_AM2J: return &g.am2j; case TC_G_AC2J: return &g.ac2j;
        case TC_G_AP2JE: return &g.ap2je; case TC_G_AM2JE: return &g.am2je; case TC_G_AC2JE: return &g.ac2je;
        case TC_G_AP3J: return &g.ap3j; case TC_G_AM3J: return &g.am3j; case TC_G_AC3J: return &g.ac3j;
        case TC_G_APPH: return &g.apph; case TC_G_AMPH: return &g.amph; case TC_G_ACPH: return &g.acph;
        case TC_G_PVOL: return &g.pvol; case TC_G_UDX2MM: return &g.udx2mm; case TC_G_UDX2CC: return &g.udx2cc;
        case TC_G_AK1: return &g.ak1;   case TC_G_AK3: return &g.ak3;
        default: return nullptr;
    }
}

}  // namespace tcgb

// ---------------------------------------------------------------------------
extern "C" {

int tc_read_bou(const char* path, tc_bou* out, char* err, int errlen) {
    auto fail = [&](int code, const std::string& m) {
        if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", m.c_str());
        return code;
    };
    if (!path || !out) return fail(2000, "null argument");
    std::ifstream f(path);
    if (!f) return fail(2001, std::string("cannot open ") + path);
    std::vector<std::string> recs;
    std::string l;
    while (std::getline(f, l)) {
        if (!l.empty() && l.back() == '\r') l.pop_back();
        recs.push_back(l);
    }
    tc_bou b;
    std::memset(&b, 0, sizeof b);
    using tcgb::Item;
    std::vector<std::vector<Item>> lists = {
        {{1, &b.nthm}, {1, &b.nzm}, {1, &b.nrm}, {1, &b.nsst}, {1, &b.idtv}, {1, &b.nread}},
        {{1, &b.ntst}, {0, &b.tout}, {0, &b.tmax}, {1, &b.ireset}, {0, &b.walltimemax}},
        {{0, &b.alx3}, {0, &b.rint}, {0, &b.rext}, {1, &b.istr}, {0, &b.str}, {0, &b.lamb}},
        {{0, &b.virotint}, {0, &b.virotext}, {0, &b.sizepert}, {0, &b.omegapert}},
        {{0, &b.ren}, {0, &b.romeg}, {0, &b.resid}, {0, &b.limitCFL}},
        {{0, &b.tsta}, {1, &b.starea}},
        {{0, &b.dtmin}, {0, &b.dtmax}, {0, &b.limitVel}, {0, &b.cfllim}},
        {{1, &b.nslabr}, {1, &b.dpthcut}, {1, &b.dpstave}, {0, &b.tframe2d}},
        {{1, &b.dpfullf}, {0, &b.tframe3d}},
        {{1, &b.minstrt}, {1, &b.minstrz}, {1, &b.multmin}},
    };
    size_t line = 0;
    for (size_t n = 0; n < lists.size(); ++n) {
        if (line >= recs.size()) return fail(2002, "bou.in ends before value record " + std::to_string(n + 1));
        ++line;  // header record, format (a4)
        std::string e;
        if (!tcgb::list_read(recs, line, lists[n], e))
            return fail(2002, "bou.in value record " + std::to_string(n + 1) + ": " + e);
    }
    *out = b;
    return 0;
}

int tc_grid_array(const tc_bou* cfg, int which, double* out, int len) {
    if (!cfg || !out) return -2000;
    tcgb::Grid g;
    std::string e = tcgb::build_grid(*cfg, g);
    if (!e.empty()) return -2003;
    const std::vector<double>* a = tcgb::grid_array(g, which);
    if (!a) return -2004;
    if ((int)a->size() > len) return -2005;
    for (size_t i = 0; i < a->size(); ++i) out[i] = (*a)[i];
    return (int)a->size();
}

const char* tc_version(void) { return "tcgb300 0.1 (sm_103a, FP64)"; }

}  // extern "C"
