/*
 * xml_io.cpp -- see xml_io.h.
 */
#include "xml_io.h"

#include <cerrno>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace pcs {

/* ======================================================================= */
/* parser                                                                  */
/* ======================================================================= */

const XmlNode* XmlNode::first_child_element(const char* n) const
{
    for (const auto& c : children)
        if (c.kind == Element && c.name == n) return &c;
    return nullptr;
}

const std::string* XmlNode::text() const
{
    if (!children.empty() && children.front().kind == Text) return &children.front().value;
    return nullptr;
}

namespace {

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

struct Parser {
    const std::string& s;
    size_t i = 0;
    explicit Parser(const std::string& src) : s(src) {}

    [[noreturn]] void fail(const char* what)
    {
        throw XmlError("error::XMLGeneric", std::string("TinyXML: LoadFile: ") + what + " at offset " + std::to_string(i));
    }
    bool starts(const char* p) const { return s.compare(i, std::strlen(p), p) == 0; }
    void skip_ws()
    {
        while (i < s.size() && is_ws(s[i])) ++i;
    }
    std::string decode(const std::string& raw)
    {
        std::string out;
        out.reserve(raw.size());
        for (size_t k = 0; k < raw.size(); ++k) {
            if (raw[k] != '&') {
                out += raw[k];
                continue;
            }
            size_t e = raw.find(';', k);
            if (e == std::string::npos) {
                out += raw[k];
                continue;
            }
            std::string ent = raw.substr(k + 1, e - k - 1);
            if (ent == "lt") out += '<';
            else if (ent == "gt") out += '>';
            else if (ent == "amp") out += '&';
            else if (ent == "quot") out += '"';
            else if (ent == "apos") out += '\'';
            else if (!ent.empty() && ent[0] == '#') {
                unsigned long cp = (ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X')) ? std::strtoul(ent.c_str() + 2, nullptr, 16)
                                                                                       : std::strtoul(ent.c_str() + 1, nullptr, 10);
                if (cp < 0x80) out += (char)cp;
                else if (cp < 0x800) {
                    out += (char)(0xC0 | (cp >> 6));
                    out += (char)(0x80 | (cp & 0x3F));
                } else if (cp < 0x10000) {
                    out += (char)(0xE0 | (cp >> 12));
                    out += (char)(0x80 | ((cp >> 6) & 0x3F));
                    out += (char)(0x80 | (cp & 0x3F));
                } else {
                    out += (char)(0xF0 | (cp >> 18));
                    out += (char)(0x80 | ((cp >> 12) & 0x3F));
                    out += (char)(0x80 | ((cp >> 6) & 0x3F));
                    out += (char)(0x80 | (cp & 0x3F));
                }
            } else {
                out += raw.substr(k, e - k + 1);
            }
            k = e;
        }
        return out;
    }
    /* parse child nodes until </name> (or end for the document) */
    void parse_children(XmlNode& parent, bool document)
    {
        for (;;) {
            size_t start = i;
            skip_ws();
            if (i >= s.size()) {
                if (document) return;
                fail("XML_ERROR_PARSING_ELEMENT (unclosed element)");
            }
            if (starts("</")) {
                if (document) fail("XML_ERROR_PARSING_ELEMENT (stray end tag)");
                i += 2;
                size_t e = s.find('>', i);
                if (e == std::string::npos) fail("XML_ERROR_PARSING_ELEMENT");
                std::string nm = s.substr(i, e - i);
                while (!nm.empty() && is_ws(nm.back())) nm.pop_back();
                if (nm != parent.name) fail("XML_ERROR_MISMATCHED_ELEMENT");
                i = e + 1;
                return;
            }
            if (starts("<?")) {
                size_t e = s.find("?>", i);
                if (e == std::string::npos) fail("XML_ERROR_PARSING_DECLARATION");
                i = e + 2;
                parent.children.push_back(XmlNode{XmlNode::Other, "", "", {}});
                continue;
            }
            if (starts("<!--")) {
                size_t e = s.find("-->", i + 4);
                if (e == std::string::npos) fail("XML_ERROR_PARSING_COMMENT");
                i = e + 3;
                parent.children.push_back(XmlNode{XmlNode::Other, "", "", {}});
                continue;
            }
            if (starts("<![CDATA[")) {
                size_t e = s.find("]]>", i + 9);
                if (e == std::string::npos) fail("XML_ERROR_PARSING_CDATA");
                parent.children.push_back(XmlNode{XmlNode::Text, "", s.substr(i + 9, e - i - 9), {}});
                i = e + 3;
                continue;
            }
            if (starts("<!")) {
                size_t e = s.find('>', i);
                if (e == std::string::npos) fail("XML_ERROR_PARSING_UNKNOWN");
                i = e + 1;
                parent.children.push_back(XmlNode{XmlNode::Other, "", "", {}});
                continue;
            }
            if (starts("<")) {
                ++i;
                XmlNode el;
                el.kind = XmlNode::Element;
                size_t n0 = i;
                while (i < s.size() && !is_ws(s[i]) && s[i] != '>' && s[i] != '/') ++i;
                el.name = s.substr(n0, i - n0);
                if (el.name.empty()) fail("XML_ERROR_PARSING_ELEMENT (empty name)");
                /* attributes: skipped (accel's files carry none) but must be well formed */
                bool self_close = false;
                for (;;) {
                    skip_ws();
                    if (i >= s.size()) fail("XML_ERROR_PARSING_ELEMENT");
                    if (s[i] == '>') {
                        ++i;
                        break;
                    }
                    if (starts("/>")) {
                        i += 2;
                        self_close = true;
                        break;
                    }
                    size_t eq = s.find('=', i);
                    if (eq == std::string::npos) fail("XML_ERROR_PARSING_ATTRIBUTE");
                    i = eq + 1;
                    skip_ws();
                    if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) fail("XML_ERROR_PARSING_ATTRIBUTE");
                    char q = s[i++];
                    size_t e = s.find(q, i);
                    if (e == std::string::npos) fail("XML_ERROR_PARSING_ATTRIBUTE");
                    i = e + 1;
                }
                if (!self_close) parse_children(el, false);
                parent.children.push_back(std::move(el));
                continue;
            }
            /* text: everything from the first character after the previous
             * node (leading whitespace included) up to the next '<' */
            size_t e = s.find('<', start);
            if (e == std::string::npos) {
                if (document) return; /* trailing text after the root */
                fail("XML_ERROR_PARSING_TEXT");
            }
            parent.children.push_back(XmlNode{XmlNode::Text, "", decode(s.substr(start, e - start)), {}});
            i = e;
        }
    }
};

} // namespace

XmlNode xml_parse(const std::string& src)
{
    std::string s = src;
    if (s.size() >= 3 && (unsigned char)s[0] == 0xEF && (unsigned char)s[1] == 0xBB && (unsigned char)s[2] == 0xBF) s.erase(0, 3);
    XmlNode doc;
    doc.kind = XmlNode::Element;
    doc.name = "#document";
    Parser p(s);
    p.parse_children(doc, true);
    bool any = false;
    for (auto& c : doc.children)
        if (c.kind == XmlNode::Element) any = true;
    if (!any) throw XmlError("error::XMLGeneric", "TinyXML: LoadFile: XML_ERROR_EMPTY_DOCUMENT");
    return doc;
}

XmlNode xml_load_file(const char* path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw XmlError("error::XMLGeneric", std::string("TinyXML: LoadFile: XML_ERROR_FILE_NOT_FOUND (") + path + ")");
    std::stringstream ss;
    ss << f.rdbuf();
    return xml_parse(ss.str());
}

/* ======================================================================= */
/* input::load                                                             */
/* ======================================================================= */

namespace {

const XmlNode* child_checked(const XmlNode* parent, const char* name)
{
    if (const XmlNode* c = parent->first_child_element(name)) return c;
    throw XmlError("error::XMLMissing", std::string("No <") + name + "> in <" + parent->name + ">");
}

const std::string& child_text(const XmlNode* parent, const char* name)
{
    const XmlNode* c = child_checked(parent, name);
    const std::string* t = c->text();
    if (!t) throw XmlError("error::XMLGeneric", std::string("no text in <") + name + "> in <" + parent->name + ">");
    return *t;
}

int64_t child_int64(const XmlNode* parent, const char* name)
{
    const XmlNode* c = child_checked(parent, name);
    const std::string* t = c->text();
    long long v = 0;
    if (!t) throw XmlError("error::XMLGeneric", std::string("TinyXML: QueryInt64Text: XML_NO_TEXT_NODE for <") + name + "> in <" + parent->name + ">");
    if (std::sscanf(t->c_str(), "%lld", &v) != 1)
        throw XmlError("error::XMLGeneric", std::string("TinyXML: QueryInt64Text: XML_CAN_NOT_CONVERT_TEXT for <") + name + "> in <" + parent->name + ">");
    return (int64_t)v;
}

double child_double(const XmlNode* parent, const char* name)
{
    const XmlNode* c = child_checked(parent, name);
    const std::string* t = c->text();
    double v = 0;
    if (!t) throw XmlError("error::XMLGeneric", std::string("TinyXML: QueryDoubleText: XML_NO_TEXT_NODE for <") + name + "> in <" + parent->name + ">");
    if (std::sscanf(t->c_str(), "%lf", &v) != 1)
        throw XmlError("error::XMLGeneric", std::string("TinyXML: QueryDoubleText: XML_CAN_NOT_CONVERT_TEXT for <") + name + "> in <" + parent->name + ">");
    return v;
}

bool child_bool(const XmlNode* parent, const char* name)
{
    const XmlNode* c = child_checked(parent, name);
    const std::string* t = c->text();
    if (!t) throw XmlError("error::XMLGeneric", std::string("TinyXML: QueryBoolText: XML_NO_TEXT_NODE for <") + name + "> in <" + parent->name + ">");
    int iv = 0;
    if (std::sscanf(t->c_str(), "%d", &iv) == 1) return iv != 0;
    if (*t == "true") return true;
    if (*t == "false") return false;
    throw XmlError("error::XMLGeneric", std::string("TinyXML: QueryBoolText: XML_CAN_NOT_CONVERT_TEXT for <") + name + "> in <" + parent->name + ">");
}

template <class Parse, class Sink>
void parse_list(const XmlNode* parent, const char* name, Parse parse, Sink sink)
{
    const std::string& txt = child_text(parent, name);
    const char* ptr = txt.c_str();
    char* next = nullptr;
    for (auto v = parse(ptr, &next); ptr != next; v = parse(ptr, &next)) {
        ptr = next;
        if (*ptr == ',') ++ptr;
        sink(v);
    }
    if (*ptr != '\0')
        throw XmlError("error::XMLParsing", std::string("Can't parse list <") + name + "> in <" + parent->name +
                                               ">. Unparsable mayhem '" + ptr + "' remains.");
}

int32_t model_from(const std::string& s, std::vector<std::string>& notes)
{
    if (s == "discrete-fixed-depth") return PCS_MODEL_DISCRETE_FIXED_DEPTH;
    if (s == "discrete-variable-depth") return PCS_MODEL_DISCRETE_VARIABLE_DEPTH;
    if (s == "discrete") {
        notes.push_back("WARNING: EModel: deprecated value \"discrete\"");
        return PCS_MODEL_DISCRETE_FIXED_DEPTH;
    }
    if (s == "lognormal") return PCS_MODEL_LOGNORMAL;
    long v = 0;
    if (std::sscanf(s.c_str(), "EModel(%ld)", &v) == 1) return (int32_t)v;
    throw XmlError("error::EnumUnknownString", "'" + s + "' is not a valid EModel");
}

int32_t weighting_from(const std::string& s)
{
    if (s == "pmc-standard") return PCS_WEIGHTING_PMC_STANDARD;
    if (s == "inverse-distance-squared") return PCS_WEIGHTING_INVERSE_DIST_SQ;
    long v = 0;
    if (std::sscanf(s.c_str(), "EWeightingScheme(%ld)", &v) == 1) return (int32_t)v;
    throw XmlError("error::EnumUnknownString", "'" + s + "' is not a valid EWeightingScheme");
}

std::pair<double, double> bounds(const XmlNode* parent, const char* pattern)
{
    char lo[64], up[64];
    std::snprintf(lo, sizeof lo, pattern, "lb");
    std::snprintf(up, sizeof up, pattern, "ub");
    const double l = child_double(parent, lo);
    const double u = child_double(parent, up);
    return {l, u};
}

} // namespace

const char* model_name(int32_t m)
{
    switch (m) {
    case PCS_MODEL_DISCRETE_FIXED_DEPTH: return "discrete-fixed-depth";
    case PCS_MODEL_DISCRETE_VARIABLE_DEPTH: return "discrete-variable-depth";
    case PCS_MODEL_LOGNORMAL: return "lognormal";
    }
    return nullptr;
}

const char* weighting_name(int32_t w)
{
    switch (w) {
    case PCS_WEIGHTING_PMC_STANDARD: return "pmc-standard";
    case PCS_WEIGHTING_INVERSE_DIST_SQ: return "inverse-distance-squared";
    }
    return nullptr;
}

InputData input_load(const char* input_path, const char* data_path)
{
    std::string dpath = data_path ? data_path : "";
    try {
        if (!input_path) throw XmlError("error::XMLGeneric", "TinyXML: LoadFile: XML_ERROR_FILE_NOT_FOUND (input)");
        XmlNode input = xml_load_file(input_path);
        const XmlNode* iroot = input.first_child_element("input");
        if (!iroot) throw XmlError("error::XMLMissing", "No <input> root element (input)");
        if (!data_path) dpath = child_text(iroot, "data_file_path");
        XmlNode data = xml_load_file(dpath.c_str());
        const XmlNode* droot = data.first_child_element("data");
        if (!droot) throw XmlError("error::XMLMissing", "No <data> root element (data)");

        InputData r;
        pcs_params_defaults(&r.params);
        pcs_params& p = r.params;
        r.data_file_path = dpath;
        std::string model;
        try {
            model = child_text(iroot, "model");
        } catch (const XmlError& e) {
            if (e.kind != "error::XMLMissing") throw;
            const XmlNode* dc = iroot->first_child_element("distribution_class");
            if (!dc || !dc->text()) throw;
            model = *dc->text();
            r.notes.push_back("WARNING: using deprecated \"distribution_class\" field");
        }
        p.model = model_from(model, r.notes);
        p.weighting_scheme = weighting_from(child_text(iroot, "weighting_scheme"));
        p.component_count = (uint32_t)child_int64(iroot, "number_of_components");
        p.kmin = (uint32_t)child_int64(iroot, "kmin");
        p.de_bin_count = (uint32_t)child_int64(iroot, "number_of_de_bins");
        p.abc_sample_count = (uint32_t)child_int64(iroot, "number_of_abc_samples");
        p.avg_trial_count = (uint32_t)child_int64(iroot, "ub_average_number_of_trials");
        p.Lx = child_double(iroot, "Lx");
        p.Ly = child_double(iroot, "Ly");
        p.Lz = child_double(iroot, "Lz");
        p.gamma_initial = child_double(iroot, "gamma_initial");
        p.delta_gamma = child_double(iroot, "delta_gamma");
        try {
            p.gamma_adaptive = child_bool(iroot, "gamma_adaptive") ? 1 : 0;
        } catch (const XmlError&) {
            r.notes.push_back("Note: <gamma_adaptive> not set/invalid (old input?); defaulting to false.");
            p.gamma_adaptive = 0;
        }
        p.ub_de = child_double(iroot, "ub_de");
        auto m = bounds(iroot, "%s_m");
        p.lb_m = m.first;
        p.ub_m = m.second;
        try {
            auto sb = bounds(iroot, "%s_s");
            p.lb_s = sb.first;
            p.ub_s = sb.second;
            r.has_s_bounds = true;
            if (p.model != PCS_MODEL_LOGNORMAL) r.notes.push_back("Note: deprecated <*_s> tags found (old input?)");
        } catch (const XmlError& e) {
            if (e.kind != "error::XMLMissing") throw;
            if (p.model == PCS_MODEL_LOGNORMAL) throw;
        }
        auto cb = bounds(iroot, "%s_c");
        p.lb_c = cb.first;
        p.ub_c = cb.second;
        auto azb = bounds(iroot, "%s_az");
        p.lb_az = azb.first;
        p.ub_az = azb.second;
        r.output_file_path = child_text(iroot, "output_file_path");

        /* extensions (absent in reference inputs; defaults keep its behaviour) */
        if (iroot->first_child_element("temperature")) p.temperature = child_double(iroot, "temperature");
        if (iroot->first_child_element("viscosity")) p.viscosity = child_double(iroot, "viscosity");
        if (iroot->first_child_element("schedule")) {
            const std::string& s = child_text(iroot, "schedule");
            if (s == "delta") p.schedule = PCS_SCHEDULE_DELTA;
            else if (s == "quantile") p.schedule = PCS_SCHEDULE_QUANTILE;
            else throw XmlError("error::EnumUnknownString", "'" + s + "' is not a valid schedule");
        }
        if (iroot->first_child_element("quantile")) p.quantile = child_double(iroot, "quantile");
        if (iroot->first_child_element("perturbation")) {
            const std::string& s = child_text(iroot, "perturbation");
            if (s == "diagonal") p.perturbation = PCS_PERTURB_DIAGONAL;
            else if (s == "cholesky") p.perturbation = PCS_PERTURB_CHOLESKY;
            else throw XmlError("error::EnumUnknownString", "'" + s + "' is not a valid perturbation");
        }
        if (iroot->first_child_element("number_of_generations"))
            p.max_generations = (uint32_t)child_int64(iroot, "number_of_generations");

        r.ax = child_double(droot, "ax");
        r.ay = child_double(droot, "ay");
        r.deltat = child_double(droot, "deltat");
        parse_list(droot, "number_of_frames", [](const char* x, char** y) { return std::strtoull(x, y, 0); },
                   [&](unsigned long long v) { r.frames.push_back(v); });
        parse_list(droot, "K", [](const char* x, char** y) { return std::strtoull(x, y, 0); },
                   [&](unsigned long long v) { r.K.push_back(v); });
        parse_list(droot, "DE", [](const char* x, char** y) { return std::strtod(x, y); },
                   [&](double v) { r.DE.push_back(v); });
        if (r.K.size() != r.DE.size())
            throw XmlError("error::XMLParsing", "<K> and <DE> have different lengths");
        return r;
    } catch (const XmlError& e) {
        throw XmlError("error::XMLLoadError", std::string("Error loading input=") + (input_path ? input_path : "(null)") +
                                                   " and data=" + dpath + " | nested " + e.what());
    }
}

/* ======================================================================= */
/* output                                                                  */
/* ======================================================================= */

namespace {
void write_list(FILE* f, const char* tag, const std::vector<double>& v)
{
    std::fprintf(f, "\t<%s>", tag);
    for (size_t i = 0; i < v.size(); ++i) {
        if (i + 1 < v.size())
            std::fprintf(f, "%.18g, ", v[i]);
        else
            std::fprintf(f, "%.18g", v[i]);
    }
    std::fprintf(f, "\t</%s>\n", tag);
}
} // namespace

void output_write(const char* path, const OutputData& o)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) throw XmlError("error::XMLGeneric", std::string("cannot open output file ") + path);
    const char* mn = model_name(o.model);
    const char* wn = weighting_name(o.weighting);
    std::fprintf(f, "<output>\n");
    if (mn)
        std::fprintf(f, "\t<model>%s</model>\n", mn);
    else
        std::fprintf(f, "\t<model>EModel(%ld)</model>\n", (long)o.model);
    if (wn)
        std::fprintf(f, "\t<weighting_scheme>%s</weighting_scheme>\n", wn);
    else
        std::fprintf(f, "\t<weighting_scheme>EWeightingScheme(%ld)</weighting_scheme>\n", (long)o.weighting);
    std::fprintf(f, "\t<number_of_abc_samples>%" PRIu64 "</number_of_abc_samples>\n", o.abc);
    std::fprintf(f, "\t<number_of_components>%" PRIu64 "</number_of_components>\n", o.C);
    std::fprintf(f, "\t<number_of_z_components>%" PRIu64 "</number_of_z_components>\n", o.Z);
    std::fprintf(f, "\n");
    std::fprintf(f, "\t<meta>\n");
    for (const auto& kv : o.meta) std::fprintf(f, "\t\t<%s>%s</%s>\n", kv.first.c_str(), kv.second.c_str(), kv.first.c_str());
    std::fprintf(f, "\t</meta>\n");
    std::fprintf(f, "\n");
    std::fprintf(f, "\t<converged>%s</converged>\n", o.converged ? "true" : "false");
    std::fprintf(f, "\t<gamma>%.18g</gamma>\n", o.gamma);
    write_list(f, "m", o.m);
    if (o.model == PCS_MODEL_LOGNORMAL) write_list(f, "s", o.s);
    write_list(f, "c", o.c);
    write_list(f, "az", o.az);
    write_list(f, "dist", o.dist);
    write_list(f, "w", o.w);
    std::fprintf(f, "</output>\n");
    std::fclose(f);
}

OutputData output_load(const char* path)
{
    try {
        XmlNode doc = xml_load_file(path);
        const XmlNode* root = doc.first_child_element("output");
        if (!root) throw XmlError("error::XMLMissing", "No <output> root element");
        OutputData o;
        std::vector<std::string> notes;
        o.model = model_from(child_text(root, "model"), notes);
        o.weighting = weighting_from(child_text(root, "weighting_scheme"));
        o.abc = (uint64_t)child_int64(root, "number_of_abc_samples");
        o.C = (uint64_t)child_int64(root, "number_of_components");
        o.Z = root->first_child_element("number_of_z_components") ? (uint64_t)child_int64(root, "number_of_z_components") : 1u;
        if (const XmlNode* meta = root->first_child_element("meta"))
            for (const auto& c : meta->children)
                if (c.kind == XmlNode::Element) o.meta.emplace_back(c.name, c.text() ? *c.text() : std::string());
        const std::string& conv = child_text(root, "converged");
        o.converged = conv == "true" || conv == "1";
        o.gamma = child_double(root, "gamma");
        auto list = [&](const char* tag, std::vector<double>& out) {
            const XmlNode* n = root->first_child_element(tag);
            if (!n) return;
            const std::string* t = n->text();
            if (!t) return;
            const char* p = t->c_str();
            char* e = nullptr;
            for (;;) {
                double v = std::strtod(p, &e);
                if (e == p) break;
                out.push_back(v);
                p = e;
                while (*p == ',' || *p == ' ') ++p;
            }
            while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p;
            if (*p) throw XmlError("error::XMLParsing", std::string("Can't parse list <") + tag + "> in <output>");
        };
        list("m", o.m);
        list("s", o.s);
        list("c", o.c);
        list("az", o.az);
        list("dist", o.dist);
        list("w", o.w);
        return o;
    } catch (const XmlError& e) {
        throw XmlError("error::XMLLoadError", std::string("Error loading '") + path + "' | nested " + e.what());
    }
}

} // namespace pcs

/* ======================================================================= */
/* C ABI                                                                   */
/* ======================================================================= */

/* The XML entry points share the error slot of capi.cpp. */
namespace pcs {
void set_last_error(const std::string& m);
}

extern "C" {

pcs_status pcs_input_load(const char* input_path, const char* data_path, pcs_input** out)
{
    if (!out) {
        pcs::set_last_error("out is NULL");
        return PCS_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    try {
        auto* in = new pcs_input;
        in->d = pcs::input_load(input_path, data_path);
        *out = in;
        pcs::set_last_error("");
        return PCS_OK;
    } catch (const pcs::XmlError& e) {
        pcs::set_last_error(e.what());
        return PCS_ERR_XML;
    } catch (const std::exception& e) {
        pcs::set_last_error(e.what());
        return PCS_ERR_XML;
    }
}

pcs_status pcs_input_free(pcs_input* in)
{
    delete in;
    return PCS_OK;
}

pcs_status pcs_input_params(const pcs_input* in, pcs_params* p, pcs_observed* obs, const char** output_file_path)
{
    if (!in) {
        pcs::set_last_error("input is NULL");
        return PCS_ERR_INVALID_ARGUMENT;
    }
    if (p) *p = in->d.params;
    if (obs) {
        obs->ax = in->d.ax;
        obs->ay = in->d.ay;
        obs->deltat = in->d.deltat;
        obs->frame_counts = in->d.frames.data();
        obs->video_count = in->d.frames.size();
        obs->K = in->d.K.data();
        obs->DE = in->d.DE.data();
        obs->track_count = in->d.K.size();
    }
    if (output_file_path) *output_file_path = in->d.output_file_path.c_str();
    return PCS_OK;
}

pcs_status pcs_output_write(const char* path, int32_t model, int32_t weighting, uint64_t abc_sample_count,
                            uint64_t component_count, uint64_t z_component_count, const pcs_output_meta* meta,
                            size_t meta_count, int converged, double gamma, const double* m, size_t nm,
                            const double* s, size_t ns, const double* c, size_t nc, const double* az, size_t naz,
                            const double* dist, size_t nd, const double* w, size_t nw)
{
    try {
        if (!path) throw pcs::XmlError("error::XMLGeneric", "path is NULL");
        pcs::OutputData o;
        o.model = model;
        o.weighting = weighting;
        o.abc = abc_sample_count;
        o.C = component_count;
        o.Z = z_component_count;
        for (size_t i = 0; i < meta_count; ++i)
            o.meta.emplace_back(meta[i].key ? meta[i].key : "", meta[i].value ? meta[i].value : "");
        o.converged = converged != 0;
        o.gamma = gamma;
        if (m) o.m.assign(m, m + nm);
        if (s) o.s.assign(s, s + ns);
        if (c) o.c.assign(c, c + nc);
        if (az) o.az.assign(az, az + naz);
        if (dist) o.dist.assign(dist, dist + nd);
        if (w) o.w.assign(w, w + nw);
        pcs::output_write(path, o);
        pcs::set_last_error("");
        return PCS_OK;
    } catch (const std::exception& e) {
        pcs::set_last_error(e.what());
        return PCS_ERR_XML;
    }
}

pcs_status pcs_output_load(const char* path, pcs_output** out)
{
    if (!out || !path) {
        pcs::set_last_error("path/out is NULL");
        return PCS_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    try {
        auto* o = new pcs_output;
        o->d = pcs::output_load(path);
        for (auto& kv : o->d.meta) o->meta_view.push_back(pcs_output_meta{kv.first.c_str(), kv.second.c_str()});
        *out = o;
        pcs::set_last_error("");
        return PCS_OK;
    } catch (const std::exception& e) {
        pcs::set_last_error(e.what());
        return PCS_ERR_XML;
    }
}

pcs_status pcs_output_free(pcs_output* o)
{
    delete o;
    return PCS_OK;
}

pcs_status pcs_output_get(const pcs_output* o, pcs_output_view* v)
{
    if (!o || !v) {
        pcs::set_last_error("output/view is NULL");
        return PCS_ERR_INVALID_ARGUMENT;
    }
    const auto& d = o->d;
    v->model = d.model;
    v->weighting = d.weighting;
    v->abc_sample_count = d.abc;
    v->component_count = d.C;
    v->z_component_count = d.Z;
    v->converged = d.converged ? 1 : 0;
    v->gamma = d.gamma;
    v->m = d.m.data();
    v->nm = d.m.size();
    v->s = d.s.data();
    v->ns = d.s.size();
    v->c = d.c.data();
    v->nc = d.c.size();
    v->az = d.az.data();
    v->naz = d.az.size();
    v->dist = d.dist.data();
    v->nd = d.dist.size();
    v->w = d.w.data();
    v->nw = d.w.size();
    v->meta_count = o->meta_view.size();
    v->meta = o->meta_view.data();
    return PCS_OK;
}

} // extern "C"
