// Helpers shared by the command-line drop-ins.
#pragma once

#include <cstdio>
#include <string>
#include <vector>

namespace crispy_cli {

// The changepoint step's cutoff file as sparsecut reads it: "%f\n" until the
// end of the file (sparsecut.cpp:333-341).  The reference loops forever on
// text that is not a number and takes an empty file as one undefined
// cutoff; both are refused here.  Returns an error text, empty on success.
inline std::string read_cutoffs(const std::string& name, std::vector<float>& out, bool echo) {
    FILE* f = std::fopen(name.c_str(), "r");
    if (!f) return "cannot open the cutoff file " + name;
    out.clear();
    for (;;) {
        float c = 0.0f;
        const int got = std::fscanf(f, "%f\n", &c);
        if (got == EOF) break;
        if (got != 1) {
            std::fclose(f);
            return name + " holds something other than a number";
        }
        out.push_back(c);
        if (echo) std::printf("%g\n", (double)c);
    }
    std::fclose(f);
    if (out.empty()) return name + " holds no cutoff";
    return "";
}

}  // namespace crispy_cli
