// case_reader.hpp -- WHFast JSON case / recovery snapshot -> flat system layout.
//
// The case format is the serde form of `WHFast` (src/integrator/whfast.rs:99-120
// of the reference) as written by src/integrator/output.rs:28-54 and read back
// by output.rs:205-241; enums are externally tagged
// ("effect": {"CentralBody": {"ConstantTimeLag": {...}}}, "evolution":
// "NonEvolving" or {"Leconte2011": 0.08}).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/posidonius_gb300.h"
#include "json.hpp"

namespace posi {

struct FlatSystem {
    int64_t n = 0;
    std::vector<int64_t> si;     // POSI_SI_COUNT
    std::vector<double> sf;      // POSI_SF_COUNT
    std::vector<int64_t> bi;     // n * POSI_BI_COUNT
    std::vector<double> bf;      // n * POSI_BF_COUNT
    std::vector<double> tables;  // evolution tables (4 * rows per evolving body)
    std::vector<double> roche;   // n * n
};

// Returns POSI_OK, POSI_ERR_PARSE (missing/ill-typed field) or
// POSI_ERR_UNSUPPORTED (a feature outside this path); err explains.
int read_case(const json::Value& doc, FlatSystem& out, std::string& err);

}  // namespace posi
