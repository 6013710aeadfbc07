/*
 * xml_io.h -- accel's file formats: input.xml + data.xml in, output.xml out.
 *
 * A small flat-XML reader written for these files (the reference parses them
 * with tinyxml2 5.0.1, external/tinyxml2): elements, attributes, comments,
 * declarations, CDATA and the five predefined entities plus character
 * references.  Text-node and number conversion follow the reference's
 * loader (src/gpu/shared/input.cpp:101-235): a text node keeps its leading
 * and trailing whitespace, integers and doubles are read with sscanf
 * ("%lld" / "%lf"), booleans accept an integer or exactly "true"/"false",
 * and lists are strtoull(.., 0) / strtod items separated by single commas
 * with nothing left over.
 */
#ifndef PCS_XML_IO_H
#define PCS_XML_IO_H

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pcs.h"

namespace pcs {

/* Error with the reference's error class name as its prefix
 * (error::XMLLoadError and subclasses, shared/errors.hpp:21-42). */
struct XmlError : std::runtime_error {
    std::string kind;
    XmlError(const std::string& k, const std::string& m) : std::runtime_error(k + ": " + m), kind(k) {}
};

struct XmlNode {
    enum Kind { Element, Text, Other } kind = Element;
    std::string name;  /* element name */
    std::string value; /* text content for Text nodes */
    std::vector<XmlNode> children;
    const XmlNode* first_child_element(const char* n) const;
    /* tinyxml2 GetText(): the first child when it is a text node, else null */
    const std::string* text() const;
};

/* parses a whole document; throws XmlError("error::XMLGeneric", ...) */
XmlNode xml_parse(const std::string& src);
XmlNode xml_load_file(const char* path);

struct InputData {
    pcs_params params{};
    double ax = 0, ay = 0, deltat = 0;
    std::vector<uint64_t> frames, K;
    std::vector<double> DE;
    std::string output_file_path;
    std::string data_file_path;
    bool has_s_bounds = false;
    std::vector<std::string> notes; /* warnings the reference prints to stderr */
};

/* input::load (shared/input.cpp:101-235) */
InputData input_load(const char* input_path, const char* data_path);

struct OutputData {
    int32_t model = 0, weighting = 0;
    uint64_t abc = 0, C = 0, Z = 0;
    std::vector<std::pair<std::string, std::string>> meta;
    bool converged = false;
    double gamma = 0;
    std::vector<double> m, s, c, az, dist, w;
};

/* output::write (shared/output.cpp:184-258); s is written for the lognormal model */
void output_write(const char* path, const OutputData& o);
OutputData output_load(const char* path);

const char* model_name(int32_t model);
const char* weighting_name(int32_t w);

} // namespace pcs

struct pcs_input {
    pcs::InputData d;
};
struct pcs_output {
    pcs::OutputData d;
    std::vector<pcs_output_meta> meta_view;
};

#endif
