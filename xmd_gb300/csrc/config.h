// config.h - YAML parameters of the hot path: parsing, merging and units.
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "../../include/xmd_gpu.h"

namespace xmdg {

// A YAML node restricted to what XMD parameter files use: block mappings,
// plain/quoted scalars, block literals (`|`, `|-`) and flow sequences.
struct YNode {
    enum Kind { Null, Scalar, Map, Seq } kind = Null;
    std::string scalar;
    std::vector<std::pair<std::string, YNode>> map;
    std::vector<YNode> seq;

    const YNode *get(const std::string &key) const;
    YNode *get_mut(const std::string &key);
};

// Throws std::runtime_error with a line number on malformed input.
YNode parse_yaml(const std::string &text);
// Recursive merge of overrides over defaults (the algorithm merge_yaml of
// src/utils/yaml.cpp:4-42 is written for).
YNode merge_yaml(const YNode &defaults, const YNode &overrides);
// The built-in defaults of the hot-path sections.
const std::string &defaults_yaml_text();

// quantity(s, def_unit): src/utils/units.cpp:12-52.  "<magnitude> <unit
// expression>" or a bare expression scaled by def_unit.
double parse_quantity(const std::string &s, double def_unit = 1.0);
double unit_value(const std::string &name);  // throws on unknown symbol

// Resolve a merged parameter tree into xmd_params (params.cpp:43-197).
void resolve_params(const YNode &root, xmd_params *out);
// Parse overrides text, merge over defaults, resolve.
void params_from_yaml(const std::string &overrides_text, xmd_params *out);

}  // namespace xmdg
