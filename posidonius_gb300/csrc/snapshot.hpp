// snapshot.hpp -- recovery snapshots and historic records of the drop-in path.
//
// Recovery snapshot (src/integrator/output.rs:28-54): the WHFast or IAS15 case document
// the run started from, with every field the integration changes replaced by
// the device state, written back as pretty-printed JSON (2-space indentation,
// as serde_json::to_string_pretty).  Fields the integrator recomputes before
// using them (heliocentric copies, alternative coordinates, effect scratch
// values) keep the values they had in the source document.
//
// Historic record (src/integrator/output.rs:91-135): per body, bincode of
// (f64 t, f64 dt, i32 id, f64 x12) then (f64 x5), little-endian: 156 bytes.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/posidonius_gb300.h"
#include "json.hpp"

namespace posi {

constexpr int kHistoryFields = 20;           // HR_* record of the kernel
constexpr int64_t kHistoryBytesPerBody = 156;  // 8 + 8 + 4 + 8 * 17

// Shortest decimal text that reads back to exactly `v` (always with a '.' or
// an exponent, so that serde reads it as a float).
std::string format_double(double v);

// Serialise with serde_json's pretty layout.
void write_json(const json::Value& v, std::string& out, int indent = 0);

// Replace the dynamic fields of a WHFast or IAS15 case document by the flat
// state of its system (n bodies; ias: the IAS15 per-body state, n x
// POSI_IAS_COUNT, for an IAS15 document).  Returns false if the document
// lacks a field.
bool update_case_document(json::Value& doc, int64_t n, const int64_t* sys_i64, const double* sys_f64,
                          const int64_t* body_i64, const double* body_f64, const double* roche, const double* ias,
                          std::string& err);

// Append the bincode bytes of one historic record of n bodies
// (records: n x kHistoryFields doubles, id stored as a double).
void encode_history_record(const double* records, int64_t n, std::vector<unsigned char>& out);

}  // namespace posi
