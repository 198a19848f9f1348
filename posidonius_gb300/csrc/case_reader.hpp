// case_reader.hpp -- WHFast / IAS15 JSON case or recovery snapshot -> flat
// system layout.
//
// The case format is the serde form of `WHFast` (src/integrator/whfast.rs:99-120
// of the reference) or of `Ias15` (src/integrator/ias15.rs:28-224) as written by src/integrator/output.rs:28-54 and read back
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
    std::vector<double> ias;     // n * POSI_IAS_COUNT (IAS15 cases; zeros otherwise)
};

// Returns POSI_OK, POSI_ERR_PARSE (missing/ill-typed field) or
// POSI_ERR_UNSUPPORTED (a feature outside this path); err explains.
int read_case(const json::Value& doc, FlatSystem& out, std::string& err);

}  // namespace posi
