/*
 * oracle_pre.cpp -- CPU restatement of CRiSPy's preprocess step
 * (src/preprocess/preprocess.cpp), end to end: records, filters, duplicate
 * merge, output files.
 *
 * TEST INFRASTRUCTURE ONLY (what tests compare crispy_preprocess and the
 * preprocess executable with; the product never links it).  It follows the
 * reference's control flow step by step, in plain C++: fgets into a
 * 4096-byte buffer, the same trims, a record list in file order, a stable
 * sort by (length, strcmp), the adjacent-duplicate fold and fprintf output.
 * Pinned against the reference's own preprocess compiled from source
 * (oracle/_ref/preprocess) by tests/test_reference_live.py and by the
 * fixtures under tests/golden/pre/.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "oracle.h"

namespace {

struct Rec {
    std::string seq, label;
    int freq;
    int order;   // position in file order (the list's insertion order)
};

// deleteSpaces (preprocess.cpp:58-64): strip trailing whitespace unless the
// string has nothing else.
void strip_ws(std::string& s) {
    const size_t k = s.find_last_not_of("\n\r \t\v\f\b");
    if (k != std::string::npos) s = s.substr(0, k + 1);
}

// deleteSpacesInSeq (preprocess.cpp:65-71): cut after the last base letter,
// unless there is none.
void strip_seq(std::string& s) {
    const size_t k = s.find_last_of("nNATGCatgc");
    if (k != std::string::npos) s = s.substr(0, k + 1);
}

// fgets whose failure leaves buf as it was (the caller then tests feof).
void next_piece(char* buf, FILE* f) {
    if (std::fgets(buf, 4096, f) == nullptr) return;
}

// READ::initialize (preprocess.cpp:33-41).
Rec make_rec(const std::string& seq, std::string label, int freq, int order) {
    std::string l;
    for (char c : label)
        if (!(c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r')) l += c;
    return Rec{seq, l, freq, order};
}

// readFile (preprocess.cpp:74-242).  Returns readIndex, or -1 (cannot open)
// / -2 (first line not a FASTA header).
int read_records(const char* path, bool fastq, std::vector<Rec>& out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return -1;
    char buf[4096];
    std::string line, seq, label;
    int index = 0;
    bool end_flag = false;
    if (!fastq) {
        if (!std::fgets(buf, sizeof buf, f)) buf[0] = '\0';
        line.assign(buf);
        if (line.empty() || line[0] != '>') { std::fclose(f); return -2; }
        strip_ws(line);
        label = line;
        while (!std::feof(f)) {
            buf[0] = '$';
            if (!std::fgets(buf, sizeof buf, f)) { /* buf keeps '$' */ }
            line.assign(buf);
            strip_ws(line);
            const char c = line.empty() ? '\0' : line[0];
            if (c != '>' && c != '$') {
                strip_seq(line);
                seq += line;
                continue;
            } else if (seq.empty()) {
                ++index;
                if (buf[0] == '$') { end_flag = true; break; }
                continue;
            } else {
                strip_seq(seq);
                out.push_back(make_rec(seq, label, 1, (int)out.size()));
                ++index;
                seq.clear();
                if (buf[0] == '$') { end_flag = true; break; }
                strip_ws(line);
                label = line;
                continue;
            }
        }
    } else {
        while (!std::feof(f)) {
            buf[0] = '$';
            next_piece(buf, f);
            line.assign(buf);
            if (std::feof(f) || buf[0] == '$') { end_flag = true; break; }
            strip_ws(line);
            label = line;
            next_piece(buf, f);
            line.assign(buf);
            if (std::feof(f) || buf[0] == '$') { end_flag = true; break; }
            strip_ws(line);
            seq = line;
            const int fr = seq.empty() ? 0 : 1;
            out.push_back(make_rec(seq, label, fr, (int)out.size()));
            ++index;
            next_piece(buf, f);
            if (std::feof(f) || buf[0] == '$') { end_flag = true; break; }
            next_piece(buf, f);
            if (std::feof(f) || buf[0] == '$') { end_flag = true; break; }
        }
    }
    if (!end_flag && !seq.empty()) {
        strip_seq(seq);
        out.push_back(make_rec(seq, label, 1, (int)out.size()));
        ++index;
    }
    std::fclose(f);
    return index;
}

// processReadLength (preprocess.cpp:322-392).
int length_filter(std::vector<Rec>& recs, double sd_allowed) {
    double sum = 0, cnt = 0;
    for (const Rec& r : recs)
        if (r.freq) { sum += r.seq.length() + 0.0; ++cnt; }
    if (cnt < 1) return 0;
    const double ave = sum / cnt;
    double acc = 0;
    int lo = 65535, hi = 0;
    for (const Rec& r : recs) {
        if (!r.freq) continue;
        const double d = r.seq.length() - ave;
        acc += d * d;
        if ((size_t)lo > r.seq.length()) lo = (int)r.seq.length();
        if ((size_t)hi < r.seq.length()) hi = (int)r.seq.length();
    }
    acc = acc / cnt;
    const double sd = std::sqrt(acc);
    const double dlo = ave - sd_allowed * sd, dhi = ave + sd_allowed * sd;
    // (int) of an out-of-range double is undefined; saturate
    const int clo = dlo >= 2147483647.0 ? 2147483647 : dlo <= -2147483648.0 ? (-2147483647 - 1) : (int)dlo;
    const int chi = dhi >= 2147483647.0 ? 2147483647 : dhi <= -2147483648.0 ? (-2147483647 - 1) : (int)dhi;
    lo = std::max(lo, clo);
    hi = std::min(hi, chi);
    int gone = 0;
    for (Rec& r : recs) {
        if (!r.freq) continue;
        if (r.seq.length() < (size_t)(long long)lo || r.seq.length() > (size_t)(long long)hi) {
            r.freq = 0;
            ++gone;
            continue;
        }
        if (r.seq.find_first_of("nN") != std::string::npos) { r.freq = 0; ++gone; }
    }
    return gone;
}

// SWLocalAlignment (preprocess.cpp:394-527) with full matrices, and the
// decision of processPrimer (:530-560): true when the read goes.
bool primer_drops(const std::string& A, const std::string& B, int max_mm) {
    const int la = (int)A.size(), lb = (int)B.size();
    std::vector<std::vector<int>> S(la + 1, std::vector<int>(lb + 1, 0)),
        ST(la + 1, std::vector<int>(lb + 1, 0)), MM(la + 1, std::vector<int>(lb + 1, 0));
    for (int i = 0; i <= la; ++i) ST[i][0] = i;
    int best = -9999, best_mm = 999, sa = 0, ea = 0;
    for (int i = 1; i <= la; ++i) {
        for (int j = 1; j <= lb; ++j) {
            const int al = A[i - 1] == B[j - 1] ? 4 : -1;
            const int c0 = S[i - 1][j - 1] + al, c1 = S[i - 1][j] - 2, c2 = S[i][j - 1] - 2;
            int v = std::max(std::max(std::max(c0, c1), c2), 0);
            S[i][j] = v;
            if (v == 0) { ST[i][j] = i - 1; MM[i][j] = 0; }
            else if (v == c0) { ST[i][j] = ST[i - 1][j - 1]; MM[i][j] = MM[i - 1][j - 1] + (al != 4); }
            else if (v == c1) { ST[i][j] = ST[i - 1][j]; MM[i][j] = MM[i - 1][j] + 1; }
            else { ST[i][j] = ST[i][j - 1]; MM[i][j] = MM[i][j - 1] + 1; }
            if (best < v || (best == v && best_mm > MM[i][j])) {
                best = v; sa = ST[i][j]; ea = i; best_mm = MM[i][j];
            }
        }
    }
    const int tot = best_mm + sa + std::abs(la - ea);
    const int s0 = tot <= max_mm ? sa : 0, e0 = tot <= max_mm ? ea : 0;
    return s0 == e0;
}

}  // namespace

extern "C" int oracle_preprocess(const char* in_path, const char* out_path, int fastq,
                                 int length_check, double sd, const char* primer, int max_mm,
                                 int64_t* counts) {
    std::vector<Rec> recs;
    const int records = read_records(in_path, fastq != 0, recs);
    if (records < 0) return records;
    int gone_len = 0, gone_primer = 0, merges = 0;
    if (length_check) gone_len = length_filter(recs, sd);
    if (primer) {
        const std::string p(primer);
        for (Rec& r : recs) {
            if (!r.freq) continue;
            const size_t take = std::min(p.size() * 2, r.seq.size());
            if (primer_drops(p, r.seq.substr(0, take), max_mm)) { r.freq = 0; ++gone_primer; }
        }
    }
    // mergeReads (preprocess.cpp:244-280): stable sort by (length, strcmp),
    // then each read equal to the next live read hands its count on
    std::stable_sort(recs.begin(), recs.end(), [](const Rec& a, const Rec& b) {
        if (a.seq.length() == b.seq.length()) return std::strcmp(a.seq.c_str(), b.seq.c_str()) < 0;
        return a.seq.length() < b.seq.length();
    });
    int prev = -1;
    for (int k = 0; k < (int)recs.size(); ++k) {
        if (!recs[k].freq) continue;
        if (prev >= 0 && recs[prev].seq == recs[k].seq) {
            recs[k].freq += recs[prev].freq;
            recs[prev].freq = 0;
            ++merges;
        }
        prev = k;
    }
    // writeToFile (preprocess.cpp:562-601)
    FILE* fo = std::fopen(out_path, "wb");
    FILE* ff = std::fopen((std::string(out_path) + ".frq").c_str(), "wb");
    if (!fo || !ff) {
        if (fo) std::fclose(fo);
        if (ff) std::fclose(ff);
        return -3;
    }
    int64_t kept = 0;
    for (const Rec& r : recs) {
        if (!r.freq) continue;
        const std::string lab = fastq ? r.label : r.label.substr(1, r.label.length() - 1);
        std::fprintf(fo, "> %s\n", lab.c_str());
        std::fprintf(ff, "%s ", lab.c_str());
        std::fprintf(fo, "%s\n", r.seq.c_str());
        std::fprintf(ff, "%d\n", r.freq);
        ++kept;
    }
    std::fclose(fo);
    std::fclose(ff);
    if (counts) {
        counts[0] = records;
        counts[1] = gone_len;
        counts[2] = gone_primer;
        counts[3] = merges;
        counts[4] = kept;
    }
    return 0;
}
