// Host-side results of a run in the reference's output formats: the per-configuration
// finalisation of the PT measurement loop (J:1542-1684), the disorder sums of Collect_data
// (J:2917-3207, serial form) and the files of Write_files (J:3210-3575): cfen, cfma, cfnm, cfst,
// cfhs, cfxy, cfnd, cfnu, cfpt, cfph.  Fixed-format records use the reference's edit descriptors
// (ES24.16, E12.6, I4, I8, I12); the header records follow gfortran's list-directed layout (a
// leading blank, integers in 12 columns, REAL(8) as G26.17E3).  FP64 throughout, no contraction.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/j1j2c.h"

namespace {

// ---- Fortran edit descriptors ---------------------------------------------------------------
std::string ld_int(long long v)  // list-directed default INTEGER: 12 columns
{
    char b[32];
    std::snprintf(b, sizeof b, "%12lld", v);
    return b;
}

// list-directed REAL(8) as gfortran writes it: G26.17E3 -- fixed form with 17 significant digits
// in 21 columns plus 5 blanks for 0.1 <= |v| < 1e17 (and 0), else 1P scientific, 3-digit exponent
std::string ld_real(double v)
{
    char b[64];
    const double a = std::fabs(v);
    if (a == 0.0 || (a >= 0.1 && a < 1e17)) {
        int k = a == 0.0 ? 1 : (int)std::floor(std::log10(a)) + 1;  // digits before the point
        char t[64];
        std::snprintf(t, sizeof t, "%.*f", 17 - k < 0 ? 0 : 17 - k, v);
        // rounding can carry into a new digit (9.99.. -> 10.0..): keep 17 significant digits
        if (a != 0.0 && std::fabs(std::atof(t)) >= std::pow(10.0, k) && 17 - k - 1 >= 0)
            std::snprintf(t, sizeof t, "%.*f", 17 - k - 1, v);
        std::snprintf(b, sizeof b, "%21s     ", t);
        return b;
    }
    char t[64];
    std::snprintf(t, sizeof t, "%.16E", v);  // d.dddE+dd
    std::string s(t);
    const size_t e = s.find('E');
    const int ex = std::atoi(s.c_str() + e + 1);
    char ebuf[16];
    std::snprintf(ebuf, sizeof ebuf, "E%c%03d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    s = s.substr(0, e) + ebuf;
    std::snprintf(b, sizeof b, "%26s", s.c_str());
    return b;
}

std::string es24_16(double v)
{
    char b[64];
    std::snprintf(b, sizeof b, "%24.16E", v);
    return b;
}

// Ew.d with w = 12, d = 6: 0.dddddd mantissa, two-digit exponent; the optional leading zero is
// dropped when the sign needs its column
std::string e12_6(double v)
{
    char t[64];
    if (v == 0.0 || !std::isfinite(v)) {
        if (v == 0.0) return "0.000000E+00";
        std::snprintf(t, sizeof t, "%12s", "************");
        return t;
    }
    std::snprintf(t, sizeof t, "%.5E", std::fabs(v));  // d.dddddE+xx: 6 significant digits
    std::string s(t);
    const size_t e = s.find('E');
    const int ex = std::atoi(s.c_str() + e + 1) + 1;
    std::string digits = s.substr(0, 1) + s.substr(2, e - 2);  // dddddd
    char out[64];
    std::snprintf(out, sizeof out, "%s.%sE%c%02d", v < 0 ? "-" : "0", digits.c_str(),
                  ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    return out;
}

std::string iw(long long v, int w)
{
    char b[32];
    std::snprintf(b, sizeof b, "%*lld", w, v);
    return b;
}

std::string text(const char* s) { return s ? std::string(s) : std::string(); }

// ---- per-configuration finalisation ---------------------------------------------------------
struct ConfSlot {  // the quantities one configuration adds per temperature slot (J:1542-1684)
    double absmag, absmag2, mag2, mag4, logmag, susc, susc2, UL, UL2, US, US2, en, en2, sph,
        sph2, str2, str4, absstr, strx, strx2, strx4, USX, USX2, stry, stry2, stry4, USY, USY2,
        absstr2, suscstr, suscstr2, nem, nem2, nbar, nbarabs, nbar_sq, nbar2, nbar4, UBN, UBN2,
        stripediff, besten, finalen;
};

struct Results {
    j1j2c_run_info info{};
    std::string impmode, start, straxis, samplermode, updateorder, tempprotocol, ptstartmode,
        ptladdermode;
    std::vector<double> temps;
    int ntemp = 0, N = 0;
    std::vector<std::vector<ConfSlot>> confs;   // per configuration, per slot
    std::vector<double> hist;                   // NTEMP x BINS, sum of conf histograms / NMESS
    std::vector<double> hist_min, hist_bin;     // of the last configuration
    std::vector<std::vector<int32_t>> flips;    // per configuration: NTEMP x N
    std::vector<std::vector<double>> phi;       // per configuration: N
    std::vector<long long> swap_att, swap_acc;  // NREPLICA - 1
    long long visit_both = 0;
};

double binder4(double m4, double m2) { return m2 > 0.0 ? 1.0 - m4 / (3.0 * m2 * m2) : 0.0; }

ConfSlot finalize_slot(const j1j2c_slot_sums& s, double beta, int nocc)
{
    const double n = (double)s.nmeasure;
    ConfSlot c{};
    const double absmag = s.absmag / n, mag2 = s.mag2 / n, mag4 = s.mag4 / n, en = s.en / n,
                 en2 = s.en2 / n;
    const double totalstrx = s.strx_abs / n, totalstry = s.stry_abs / n;
    const double strx2 = s.strx2 / n, strx4 = s.strx4 / n, stry2 = s.stry2 / n,
                 stry4 = s.stry4 / n, str2 = s.str2 / n, str4 = s.str4 / n,
                 absstr = s.absstr / n, nem = s.nem / n, nbar = s.nbar / n,
                 nbarabs = s.nbarabs / n, nbar2 = s.nbar2 / n, nbar4 = s.nbar4 / n;
    const double suscabs = (mag2 - absmag * absmag) * (double)nocc * beta;
    const double susstrip = (str2 - absstr * absstr) * (double)nocc * beta;
    const double UL = binder4(mag4, mag2);
    const double US = str2 > 0.0 ? 2.0 - str4 / (str2 * str2) : 0.0;
    const double USX = binder4(strx4, strx2), USY = binder4(stry4, stry2);
    const double UBN = binder4(nbar4, nbar2);
    const double sph = (en2 - en * en) * (double)nocc * (beta * beta);  // ...*beta**2
    c.absmag = absmag;
    c.absmag2 = absmag * absmag;
    c.mag2 = mag2;
    c.mag4 = mag4;
    c.logmag = absmag > 0.0 ? std::log(absmag) : std::log(2.2250738585072014e-308);
    c.susc = suscabs;
    c.susc2 = suscabs * suscabs;
    c.UL = UL;
    c.UL2 = UL * UL;
    c.US = US;
    c.US2 = US * US;
    c.en = en;
    c.en2 = en * en;
    c.sph = sph;
    c.sph2 = sph * sph;
    c.str2 = str2;
    c.str4 = str4;
    c.absstr = absstr;
    c.strx = totalstrx;
    c.strx2 = strx2;
    c.strx4 = strx4;
    c.USX = USX;
    c.USX2 = USX * USX;
    c.stry = totalstry;
    c.stry2 = stry2;
    c.stry4 = stry4;
    c.USY = USY;
    c.USY2 = USY * USY;
    c.absstr2 = absstr * absstr;
    c.suscstr = susstrip;
    c.suscstr2 = susstrip * susstrip;
    c.nem = nem;
    c.nem2 = nem * nem;
    c.nbar = nbar;
    c.nbarabs = nbarabs;
    c.nbar_sq = nbar * nbar;
    c.nbar2 = nbar2;
    c.nbar4 = nbar4;
    c.UBN = UBN;
    c.UBN2 = UBN * UBN;
    c.stripediff = totalstrx * totalstrx - totalstry * totalstry;
    c.besten = s.best_en;
    c.finalen = s.final_en;
    return c;
}

double coexistence_angle(double x, double y)  // Stripe_coexistence_angle (J:1051-1063)
{
    const double d = x * x + y * y;
    return d > 0.0 ? 4.0 * x * x * y * y / (d * d) : 0.0;
}

// disorder average of one member over the processed configurations, and its error
struct Avg {
    const Results& r;
    int t;
    double mean(double ConfSlot::*m) const
    {
        double s = 0.0;
        for (const auto& c : r.confs) s += c[t].*m;
        return s / (double)r.confs.size();
    }
    double err(double ConfSlot::*m, double ConfSlot::*m2) const  // sqrt([x^2] - [x]^2)/sqrt(n)
    {
        const double f = (double)r.confs.size(), a = mean(m), b = mean(m2);
        return std::sqrt(b - a * a) / std::sqrt(1.0 * f);
    }
};

std::string file_name(const char* stem, int L, int H)
{
    char b[64];
    std::snprintf(b, sizeof b, "%s%04d%04d.dat", stem, L, H);
    return b;
}

void header(FILE* f, const Results& r, const char* size_label, bool full, bool energy)
{
    const j1j2c_run_info& in = r.info;
    std::fprintf(f, " program J1J2_6          \n");
    if (size_label) std::fprintf(f, " %s%s\n", size_label, ld_int(in.L).c_str());
    std::fprintf(f, " J1                      %s\n", ld_real(in.J1).c_str());
    std::fprintf(f, " deltaJ1                 %s\n", ld_real(in.deltaJ1).c_str());
    std::fprintf(f, " J2                      %s\n", ld_real(in.J2).c_str());
    std::fprintf(f, " J3                      %s\n", ld_real(in.J3).c_str());
    std::fprintf(f, " phi, xi                     %s%s\n", ld_real(in.phi).c_str(),
                 ld_real(in.xi).c_str());
    std::fprintf(f, " impurity conc.          %s\n", ld_real(in.pp).c_str());
    if (full) {
        std::fprintf(f, " impurity mode           %s\n", r.impmode.c_str());
        std::fprintf(f, " start                   %s\n", r.start.c_str());
        std::fprintf(f, " stripe axis             %s\n", r.straxis.c_str());
        std::fprintf(f, " sampler mode            %s\n", r.samplermode.c_str());
        std::fprintf(f, " update order            %s\n", r.updateorder.c_str());
        std::fprintf(f, " temperature protocol    %s\n", r.tempprotocol.c_str());
        std::fprintf(f, " PT start mode           %s\n", r.ptstartmode.c_str());
        std::fprintf(f, " PT ladder mode          %s\n", r.ptladdermode.c_str());
        std::fprintf(f, " PT replicas             %s\n", ld_int(in.nreplica).c_str());
        std::fprintf(f, " PT swap every           %s\n", ld_int(in.ptswapever).c_str());
        std::fprintf(f, " PT measure index        %s\n", ld_int(in.ptmeasindex).c_str());
        std::fprintf(f, " disorder configurations %s\n", ld_int(in.nconf).c_str());
        std::fprintf(f, " equilibration steps     %s\n", ld_int(in.neq).c_str());
        std::fprintf(f, " measurement steps       %s\n", ld_int(in.nmess).c_str());
        std::fprintf(f, " RNG seed                %s\n", ld_int(in.irinit).c_str());
        if (r.ptladdermode.rfind("SPLIT", 0) == 0) {
            std::fprintf(f, " T ladder midpoint       %s\n", ld_real(in.tladdermid).c_str());
            std::fprintf(f, " T ladder low-T fraction %s\n", ld_real(in.tladderfrac).c_str());
        }
    } else if (r.ptladdermode.rfind("SPLIT", 0) == 0) {
        std::fprintf(f, " T ladder low-T fraction %s\n", ld_real(in.tladderfrac).c_str());
    }
    if (energy) std::fprintf(f, " energy definition       exchange + phi\n");
}

}  // namespace

extern "C" {

int j1j2c_results_create(void** res, const j1j2c_run_info* info, const double* temps)
{
    if (!res || !info || !temps || info->nreplica < 1 || info->L < 1 || info->H < 1)
        return J1J2C_EINVAL;
    Results* r = new Results();
    r->info = *info;
    r->impmode = text(info->impmode);
    r->start = text(info->start);
    r->straxis = text(info->straxis);
    r->samplermode = text(info->samplermode);
    r->updateorder = text(info->updateorder);
    r->tempprotocol = text(info->tempprotocol);
    r->ptstartmode = text(info->ptstartmode);
    r->ptladdermode = text(info->ptladdermode);
    r->ntemp = info->nreplica;
    r->N = info->L * info->L * info->H;
    r->temps.assign(temps, temps + r->ntemp);
    if (info->bins > 0) {
        r->hist.assign((size_t)r->ntemp * info->bins, 0.0);
        r->hist_min.assign(r->ntemp, 0.0);
        r->hist_bin.assign(r->ntemp, 0.0);
    }
    r->swap_att.assign(r->ntemp > 1 ? r->ntemp - 1 : 0, 0);
    r->swap_acc.assign(r->ntemp > 1 ? r->ntemp - 1 : 0, 0);
    *res = r;
    return J1J2C_OK;
}

int j1j2c_results_add_conf(void* res, const j1j2c_slot_sums* sums, int32_t nocc,
                           const int64_t* swap_attempts, const int64_t* swap_accepts,
                           int32_t visited_both, const double* hist_counts,
                           const double* hist_min, const double* hist_bin,
                           const int32_t* flip_counts, const double* p)
{
    if (!res || !sums || nocc < 1) return J1J2C_EINVAL;
    Results* r = static_cast<Results*>(res);
    std::vector<ConfSlot> cs(r->ntemp);
    for (int t = 0; t < r->ntemp; ++t) {
        if (sums[t].nmeasure < 1) return J1J2C_EINVAL;
        cs[t] = finalize_slot(sums[t], 1.0 / r->temps[t], nocc);
    }
    r->confs.push_back(cs);
    const int bins = r->info.bins;
    if (bins > 0 && hist_counts) {
        for (int t = 0; t < r->ntemp; ++t) {
            const double nm = (double)sums[t].nmeasure;  // confhist / NMESS (J:1680-1682)
            for (int b = 0; b < bins; ++b)
                r->hist[(size_t)t * bins + b] += hist_counts[(size_t)t * bins + b] / nm;
            if (hist_min) r->hist_min[t] = hist_min[t];
            if (hist_bin) r->hist_bin[t] = hist_bin[t];
        }
    }
    if (flip_counts)
        r->flips.emplace_back(flip_counts, flip_counts + (size_t)r->ntemp * r->N);
    if (p) r->phi.emplace_back(p, p + r->N);
    for (size_t k = 0; k < r->swap_att.size(); ++k) {
        if (swap_attempts) r->swap_att[k] += swap_attempts[k];
        if (swap_accepts) r->swap_acc[k] += swap_accepts[k];
    }
    r->visit_both += visited_both;
    return J1J2C_OK;
}

int j1j2c_results_write(void* res, const char* dir)
{
    if (!res || !dir) return J1J2C_EINVAL;
    const Results& r = *static_cast<Results*>(res);
    const int nf = (int)r.confs.size();
    if (nf < 1) return J1J2C_ESTATE;
    const j1j2c_run_info& in = r.info;
    const double fn = (double)nf;
    auto open = [&](const char* stem) {
        const std::string path = std::string(dir) + "/" + file_name(stem, in.L, in.H);
        return std::fopen(path.c_str(), "w");
    };
    FILE* f;
    // cfen: energy and specific heat (J:3221-3258)
    if (!(f = open("cfen"))) return J1J2C_EINVAL;
    header(f, r, "linear system size      ", true, true);
    std::fprintf(f, " -------------------------\n");
    std::fprintf(f, " disorder configurations processed %s\n", ld_int(nf).c_str());
    std::fprintf(f, "    T      [<energy>]      std.en/sqrt(iconf)      [<spec.heat>]      "
                    "std.spec.heat/sqrt(iconf)   \n");
    for (int t = 0; t < r.ntemp; ++t) {
        const Avg a{r, t};
        std::fprintf(f, " %s %s %s %s %s\n", es24_16(r.temps[t]).c_str(),
                     es24_16(a.mean(&ConfSlot::en)).c_str(),
                     es24_16(a.err(&ConfSlot::en, &ConfSlot::en2)).c_str(),
                     es24_16(a.mean(&ConfSlot::sph)).c_str(),
                     es24_16(a.err(&ConfSlot::sph, &ConfSlot::sph2)).c_str());
    }
    std::fclose(f);
    // cfma: magnetisation, susceptibility, Binder (J:3263-3303)
    if (!(f = open("cfma"))) return J1J2C_EINVAL;
    header(f, r, "spatial system size     ", true, false);
    std::fprintf(f, " ------------------------\n");
    std::fprintf(f, " disorder configurations processed %s\n", ld_int(nf).c_str());
    std::fprintf(f, "    T      [<mag>]      [<mag>^2]      std.mag/sqrt(iconf)      [<susc>] .     "
                    "std.susc/sqrt(iconf)      [<Binder>]      std.bin/sqrt(iconf) [log <mag>]  "
                    "Global.Binder\n");
    for (int t = 0; t < r.ntemp; ++t) {
        const Avg a{r, t};
        const double m2 = a.mean(&ConfSlot::mag2), m4 = a.mean(&ConfSlot::mag4);
        std::string line = " ";
        for (double v : {r.temps[t], a.mean(&ConfSlot::absmag), a.mean(&ConfSlot::absmag2),
                         a.err(&ConfSlot::absmag, &ConfSlot::absmag2), a.mean(&ConfSlot::susc),
                         a.err(&ConfSlot::susc, &ConfSlot::susc2), a.mean(&ConfSlot::UL),
                         a.err(&ConfSlot::UL, &ConfSlot::UL2), a.mean(&ConfSlot::logmag),
                         1.0 - m4 / (3.0 * m2 * m2)})
            line += e12_6(v) + " ";
        line.pop_back();
        std::fprintf(f, "%s\n", line.c_str());
    }
    std::fclose(f);
    // cfnm: nematic order nbar (J:3307-3361)
    if (!(f = open("cfnm"))) return J1J2C_EINVAL;
    header(f, r, "spatial system size     ", true, false);
    std::fprintf(f, " ------------------------\n");
    std::fprintf(f, " disorder configurations processed %s\n", ld_int(nf).c_str());
    std::fprintf(f, "    T      [<n>]      [|<n>|]      [<|n|>]      [<n>].Error      "
                    "[|<n>|].Error      [<|n|>].Error      [<n^2>]      [<n^4>]      "
                    "Global.Nematic.Binder      Nematic.Binder      Nematic.Binder.Error\n");
    for (int t = 0; t < r.ntemp; ++t) {
        const Avg a{r, t};
        const double n2 = a.mean(&ConfSlot::nbar2), n4 = a.mean(&ConfSlot::nbar4);
        const double UBN = n2 > 0.0 ? 1.0 - n4 / (3.0 * n2 * n2) : 0.0;
        const double nb = a.mean(&ConfSlot::nbar), nbq = a.mean(&ConfSlot::nbar_sq);
        const double nbarerr = std::sqrt(std::fmax(0.0, nbq - nb * nb)) / std::sqrt(1.0 * fn);
        double mabs = 0.0;
        for (const auto& c : r.confs) mabs += std::fabs(c[t].nbar);
        mabs /= fn;
        double v1 = 0.0, v2 = 0.0;
        const double nabs = a.mean(&ConfSlot::nbarabs);
        for (const auto& c : r.confs) {
            v1 += (std::fabs(c[t].nbar) - mabs) * (std::fabs(c[t].nbar) - mabs);
            v2 += (c[t].nbarabs - nabs) * (c[t].nbarabs - nabs);
        }
        const double mabserr = std::sqrt(std::fmax(0.0, v1 / fn)) / std::sqrt(1.0 * fn);
        const double nabserr = std::sqrt(std::fmax(0.0, v2 / fn)) / std::sqrt(1.0 * fn);
        std::string line = " ";
        for (double v : {r.temps[t], nb, mabs, nabs, nbarerr, mabserr, nabserr, n2, n4, UBN,
                         a.mean(&ConfSlot::UBN), a.err(&ConfSlot::UBN, &ConfSlot::UBN2)})
            line += e12_6(v) + " ";
        line.pop_back();
        std::fprintf(f, "%s\n", line.c_str());
    }
    std::fclose(f);
    // cfst: stripe order, coexistence (J:3365-3436)
    if (!(f = open("cfst"))) return J1J2C_EINVAL;
    header(f, r, nullptr, false, false);
    std::fprintf(f, " ------------------------\n");
    std::fprintf(f, " disorder configurations processed %s\n", ld_int(nf).c_str());
    std::fprintf(f, "    T      absstr    str2      str4      nem      Global.Strip.Binder      "
                    "Strip.susc  Local.Strip.Binder     Local.Strip.Binder.Error      "
                    "Strip.OP.error      stri.susc.error strx   strx2   strx4   Local.Strx.Binder"
                    "    Local.Strx.Binder.Error  stry   stry2   stry4   Local.Stry.Binder    "
                    "Local.Stry.Binder.Error absstrx_absstry  absstrx_absstry.Error  coex_angle  "
                    "coex_angle.Error\n");
    for (int t = 0; t < r.ntemp; ++t) {
        const Avg a{r, t};
        double cp = 0.0, cp2 = 0.0, ca = 0.0, ca2 = 0.0;
        for (const auto& c : r.confs) {
            const double pr = c[t].strx * c[t].stry, an = coexistence_angle(c[t].strx, c[t].stry);
            cp += pr;
            cp2 += pr * pr;
            ca += an;
            ca2 += an * an;
        }
        const double s2 = a.mean(&ConfSlot::str2), s4 = a.mean(&ConfSlot::str4);
        std::string line = " ";
        for (double v : {r.temps[t], a.mean(&ConfSlot::absstr), s2, s4, a.mean(&ConfSlot::nem),
                         2.0 - s4 / (s2 * s2), a.mean(&ConfSlot::suscstr), a.mean(&ConfSlot::US),
                         a.err(&ConfSlot::US, &ConfSlot::US2),
                         a.err(&ConfSlot::absstr, &ConfSlot::absstr2),
                         a.err(&ConfSlot::suscstr, &ConfSlot::suscstr2), a.mean(&ConfSlot::strx),
                         a.mean(&ConfSlot::strx2), a.mean(&ConfSlot::strx4), a.mean(&ConfSlot::USX),
                         a.err(&ConfSlot::USX, &ConfSlot::USX2), a.mean(&ConfSlot::stry),
                         a.mean(&ConfSlot::stry2), a.mean(&ConfSlot::stry4), a.mean(&ConfSlot::USY),
                         a.err(&ConfSlot::USY, &ConfSlot::USY2), cp / fn,
                         std::sqrt(cp2 / fn - (cp / fn) * (cp / fn)) / std::sqrt(1.0 * fn), ca / fn,
                         std::sqrt(ca2 / fn - (ca / fn) * (ca / fn)) / std::sqrt(1.0 * fn)})
            line += e12_6(v) + " ";
        line.pop_back();
        std::fprintf(f, "%s\n", line.c_str());
    }
    std::fclose(f);
    // cfhs: energy histograms (J:3442-3487)
    if (in.bins > 0) {
        if (!(f = open("cfhs"))) return J1J2C_EINVAL;
        std::fprintf(f, " program J1J2_6          \n");
        std::fprintf(f, " J1                      %s\n", ld_real(in.J1).c_str());
        std::fprintf(f, " deltaJ1                 %s\n", ld_real(in.deltaJ1).c_str());
        std::fprintf(f, " J2                      %s\n", ld_real(in.J2).c_str());
        std::fprintf(f, " J3                      %s\n", ld_real(in.J3).c_str());
        std::fprintf(f, " phi                     %s\n", ld_real(in.phi).c_str());
        std::fprintf(f, " impurity conc.          %s\n", ld_real(in.pp).c_str());
        if (r.ptladdermode.rfind("SPLIT", 0) == 0)
            std::fprintf(f, " T ladder low-T fraction %s\n", ld_real(in.tladderfrac).c_str());
        std::fprintf(f, " energy definition       exchange + phi\n");
        std::fprintf(f, " -------------------------\n");
        std::fprintf(f, " disorder configurations processed %s\n", ld_int(nf).c_str());
        std::fprintf(f, " T  BIN   [<energy>]  freq\n");
        for (int t = 0; t < r.ntemp; ++t)
            for (int b = 1; b <= in.bins - 1; ++b)
                std::fprintf(f, " %s %s %s %s\n", e12_6(r.temps[t]).c_str(), iw(b, 4).c_str(),
                             e12_6(r.hist_min[t] + r.hist_bin[t] * (double)(b - 1)).c_str(),
                             e12_6(r.hist[(size_t)t * in.bins + b - 1] / fn).c_str());
        std::fclose(f);
    }
    // cfxy: per-configuration stripe data (J:3489-3503)
    if (in.write_strip) {
        if (!(f = open("cfxy"))) return J1J2C_EINVAL;
        std::fprintf(f, " iconf, T, strx, stry, absstr, D, best_en, final_en, absstrx_absstry, "
                        "coex_angle\n");
        for (int id = 0; id < nf; ++id)
            for (int t = 0; t < r.ntemp; ++t) {
                const ConfSlot& c = r.confs[id][t];
                std::string line = iw(id + 1, 4) + " ";
                for (double v : {r.temps[t], c.strx, c.stry, c.absstr, c.stripediff, c.besten,
                                 c.finalen, c.strx * c.stry, coexistence_angle(c.strx, c.stry)})
                    line += e12_6(v) + " ";
                line.pop_back();
                std::fprintf(f, "%s\n", line.c_str());
            }
        std::fclose(f);
    }
    // cfnd: per-configuration nematic data (J:3505-3516)
    if (!(f = open("cfnd"))) return J1J2C_EINVAL;
    std::fprintf(f, " iconf, T, nbar, abs_nbar, nbar2, nbar4, nbinder\n");
    for (int id = 0; id < nf; ++id)
        for (int t = 0; t < r.ntemp; ++t) {
            const ConfSlot& c = r.confs[id][t];
            std::string line = iw(id + 1, 4) + " ";
            for (double v : {r.temps[t], c.nbar, c.nbarabs, c.nbar2, c.nbar4, c.UBN})
                line += e12_6(v) + " ";
            line.pop_back();
            std::fprintf(f, "%s\n", line.c_str());
        }
    std::fclose(f);
    // cfnu: flip counts per site (J:3519-3533)
    if (in.write_numflips && !r.flips.empty()) {
        if (!(f = open("cfnu"))) return J1J2C_EINVAL;
        std::fprintf(f, " iconf, T, isite, numflips\n");
        for (size_t id = 0; id < r.flips.size(); ++id)
            for (int t = 0; t < r.ntemp; ++t)
                for (int s = 0; s < r.N; ++s)
                    std::fprintf(f, "%s %s %s %s\n", iw((long long)id + 1, 4).c_str(),
                                 e12_6(r.temps[t]).c_str(), iw(s, 8).c_str(),
                                 iw(r.flips[id][(size_t)t * r.N + s], 8).c_str());
        std::fclose(f);
    }
    // cfpt: swap statistics (J:3535-3554)
    if (r.samplermode.rfind("PT", 0) == 0) {
        if (!(f = open("cfpt"))) return J1J2C_EINVAL;
        std::fprintf(f, " pair, T_low, T_high, attempts, accepts, acceptance\n");
        for (int k = 0; k + 1 < r.ntemp; ++k) {
            const long long at = r.swap_att[k], ac = at > 0 ? r.swap_acc[k] : 0;
            std::fprintf(f, "%s %s %s %s %s %s\n", iw(k + 1, 4).c_str(), e12_6(r.temps[k]).c_str(),
                         e12_6(r.temps[k + 1]).c_str(), iw(at, 12).c_str(), iw(ac, 12).c_str(),
                         e12_6(at > 0 ? (double)ac / (double)at : 0.0).c_str());
        }
        const long long denom = (long long)nf * in.nreplica;
        std::fprintf(f, " replicas_visiting_both_extremes %s%s\n", ld_int(r.visit_both).c_str(),
                     ld_real((double)r.visit_both / (double)(denom > 1 ? denom : 1)).c_str());
        std::fclose(f);
    }
    // cfph: the random field of every configuration (J:3556-3569)
    if (in.write_phitable && !r.phi.empty()) {
        if (!(f = open("cfph"))) return J1J2C_EINVAL;
        std::fprintf(f, " iconf, isite, p\n");
        for (size_t id = 0; id < r.phi.size(); ++id)
            for (int s = 0; s < r.N; ++s)
                std::fprintf(f, "%s %s %s\n", iw((long long)id + 1, 4).c_str(), iw(s, 8).c_str(),
                             e12_6(r.phi[id][s]).c_str());
        std::fclose(f);
    }
    return J1J2C_OK;
}

void j1j2c_results_destroy(void* res) { delete static_cast<Results*>(res); }

}  // extern "C"
