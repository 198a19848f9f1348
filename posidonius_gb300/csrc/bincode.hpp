// bincode.hpp -- binary recovery snapshots of the drop-in path.
//
// The reference writes a recovery snapshot as JSON when its path ends in
// ".json" and as bincode (the bincode 1.3 crate, default options) otherwise
// (src/integrator/output.rs:28-54), and restores it the same way, trying
// WHFast, then Ias15 (:243-279).  This codec converts between the bincode
// form and the JSON document this library already reads and writes
// (json.hpp, case_reader.cpp, snapshot.cpp), so a binary snapshot takes the
// JSON path in between.
//
// bincode 1.3 with serde derive: struct fields in declaration order with no
// names; f64 and integers little-endian at their declared width (usize and
// u64: 8 bytes); bool one byte; enum variants a u32 index (declaration
// order) followed by the payload; Vec and map: a u64 length, then the
// elements (map: key, value pairs); fixed arrays ([T; N], also through
// serde-big-array): the N elements with no length.  The JSON side is
// serde_json's: an enum's unit variant is its name as a string, a newtype
// variant {"Name": value}; map keys are strings; a NaN float is null.
#pragma once
#include <string>

#include "json.hpp"

namespace posi {

// JSON document of a WHFast or Ias15 case -> bincode bytes.  The integrator
// is recognised by the document's fields.
bool json_to_bincode(const json::Value& doc, std::string& out, std::string& err);

// bincode bytes -> JSON document (members in declaration order): decoded as
// WHFast, and if that does not consume the bytes exactly, as Ias15.
bool bincode_to_json(const std::string& bytes, json::Value& doc, std::string& err);

// True when the reference would take `path` for bincode (its extension is
// not "json").
bool is_bincode_path(const std::string& path);

}  // namespace posi
