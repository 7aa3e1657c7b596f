// Import of the reference's JSON asset descriptions (host C++, no CUDA): materials and scenes.
//
// sel_material_from_json restates ImportMaterial (Source/Core/BuildCommon/ImportMaterial.cpp:56-88) followed by
// BuildMaterial (Source/Core/BuildCommon/BuildModel.cpp:22-64); sel_disney_materials_from_json restates
// ImportDisneyMaterials (ImportMaterial.cpp:91-146), the Disney-island materials file, with the same
// BuildMaterial; sel_scene_description_from_json restates ParseSceneFile
// (Source/Core/BuildCommon/CSceneBuildProcessor.cpp:32-63).  The reference reads the files with rapidjson; a
// small recursive-descent JSON reader of our own takes its place here (objects, arrays, strings with escapes,
// numbers through strtod, true / false / null).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "capi_internal.h"

namespace sel {
namespace {

struct JValue {
    enum Kind { kNull, kBool, kNumber, kString, kArray, kObject } kind = kNull;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JValue> items;                          // array elements
    std::vector<std::pair<std::string, JValue>> members;  // object members in document order

    const JValue* member(const char* name) const {
        if (kind != kObject) return nullptr;
        for (const auto& m : members)
            if (m.first == name) return &m.second;
        return nullptr;
    }
};

class JReader {
public:
    explicit JReader(const char* text) : p_(text), begin_(text) {}

    bool parse(JValue& out, std::string& error) {
        if (!value(out, 0)) {
            error = error_ + " at offset " + std::to_string(p_ - begin_);
            return false;
        }
        skip();
        if (*p_ != '\0') {
            error = "trailing characters at offset " + std::to_string(p_ - begin_);
            return false;
        }
        return true;
    }

private:
    static constexpr int kMaxDepth = 64;
    const char* p_;
    const char* begin_;
    std::string error_;

    void skip() {
        while (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r') ++p_;
    }
    bool fail(const char* what) {
        error_ = what;
        return false;
    }
    bool literal(const char* word) {
        const size_t n = std::strlen(word);
        if (std::strncmp(p_, word, n) != 0) return fail("unknown literal");
        p_ += n;
        return true;
    }
    static void put_utf8(std::string& s, uint32_t c) {
        if (c < 0x80) {
            s += char(c);
        } else if (c < 0x800) {
            s += char(0xc0 | (c >> 6));
            s += char(0x80 | (c & 0x3f));
        } else if (c < 0x10000) {
            s += char(0xe0 | (c >> 12));
            s += char(0x80 | ((c >> 6) & 0x3f));
            s += char(0x80 | (c & 0x3f));
        } else {
            s += char(0xf0 | (c >> 18));
            s += char(0x80 | ((c >> 12) & 0x3f));
            s += char(0x80 | ((c >> 6) & 0x3f));
            s += char(0x80 | (c & 0x3f));
        }
    }
    bool hex4(uint32_t& c) {
        c = 0;
        for (int k = 0; k < 4; ++k) {
            const char h = *p_++;
            c <<= 4;
            if (h >= '0' && h <= '9') c |= uint32_t(h - '0');
            else if (h >= 'a' && h <= 'f') c |= uint32_t(h - 'a' + 10);
            else if (h >= 'A' && h <= 'F') c |= uint32_t(h - 'A' + 10);
            else return fail("bad \\u escape");
        }
        return true;
    }
    bool string(std::string& s) {
        if (*p_ != '"') return fail("expected a string");
        ++p_;
        s.clear();
        for (;;) {
            const char ch = *p_;
            if (ch == '\0') return fail("unterminated string");
            if (static_cast<unsigned char>(ch) < 0x20) return fail("control character in a string");
            ++p_;
            if (ch == '"') return true;
            if (ch != '\\') {
                s += ch;
                continue;
            }
            const char e = *p_++;
            switch (e) {
                case '"': s += '"'; break;
                case '\\': s += '\\'; break;
                case '/': s += '/'; break;
                case 'b': s += '\b'; break;
                case 'f': s += '\f'; break;
                case 'n': s += '\n'; break;
                case 'r': s += '\r'; break;
                case 't': s += '\t'; break;
                case 'u': {
                    uint32_t c;
                    if (!hex4(c)) return false;
                    if (c >= 0xd800 && c < 0xdc00 && p_[0] == '\\' && p_[1] == 'u') {  // surrogate pair
                        p_ += 2;
                        uint32_t lo;
                        if (!hex4(lo)) return false;
                        if (lo < 0xdc00 || lo >= 0xe000) return fail("bad surrogate pair");
                        c = 0x10000 + ((c - 0xd800) << 10) + (lo - 0xdc00);
                    }
                    put_utf8(s, c);
                    break;
                }
                default: return fail("bad escape");
            }
        }
    }
    bool number(double& d) {
        const char* start = p_;
        if (*p_ == '-') ++p_;
        if (!std::isdigit(static_cast<unsigned char>(*p_))) return fail("bad number");
        while (std::isdigit(static_cast<unsigned char>(*p_))) ++p_;
        if (*p_ == '.') {
            ++p_;
            if (!std::isdigit(static_cast<unsigned char>(*p_))) return fail("bad number");
            while (std::isdigit(static_cast<unsigned char>(*p_))) ++p_;
        }
        if (*p_ == 'e' || *p_ == 'E') {
            ++p_;
            if (*p_ == '+' || *p_ == '-') ++p_;
            if (!std::isdigit(static_cast<unsigned char>(*p_))) return fail("bad number");
            while (std::isdigit(static_cast<unsigned char>(*p_))) ++p_;
        }
        d = std::strtod(std::string(start, p_).c_str(), nullptr);
        return true;
    }
    bool value(JValue& v, int depth) {
        if (depth > kMaxDepth) return fail("nesting too deep");
        skip();
        switch (*p_) {
            case '{': {
                ++p_;
                v.kind = JValue::kObject;
                skip();
                if (*p_ == '}') {
                    ++p_;
                    return true;
                }
                for (;;) {
                    skip();
                    std::string key;
                    if (!string(key)) return false;
                    skip();
                    if (*p_ != ':') return fail("expected ':'");
                    ++p_;
                    v.members.emplace_back(std::move(key), JValue());
                    if (!value(v.members.back().second, depth + 1)) return false;
                    skip();
                    if (*p_ == ',') {
                        ++p_;
                        continue;
                    }
                    if (*p_ == '}') {
                        ++p_;
                        return true;
                    }
                    return fail("expected ',' or '}'");
                }
            }
            case '[': {
                ++p_;
                v.kind = JValue::kArray;
                skip();
                if (*p_ == ']') {
                    ++p_;
                    return true;
                }
                for (;;) {
                    v.items.emplace_back();
                    if (!value(v.items.back(), depth + 1)) return false;
                    skip();
                    if (*p_ == ',') {
                        ++p_;
                        continue;
                    }
                    if (*p_ == ']') {
                        ++p_;
                        return true;
                    }
                    return fail("expected ',' or ']'");
                }
            }
            case '"':
                v.kind = JValue::kString;
                return string(v.str);
            case 't':
                v.kind = JValue::kBool;
                v.b = true;
                return literal("true");
            case 'f':
                v.kind = JValue::kBool;
                v.b = false;
                return literal("false");
            case 'n':
                v.kind = JValue::kNull;
                return literal("null");
            default:
                v.kind = JValue::kNumber;
                return number(v.num);
        }
    }
};

// Json::ReadFloat / ReadFloat3 / ReadBool (UtilityLib/JsonUtilities.cpp:83-97,121-140,164-182): the value when
// the member exists with the expected type (a number within float range; an array of at least three numbers, the
// first three taken), else the default.
bool float_number(const JValue& v) { return v.kind == JValue::kNumber && std::fabs(v.num) <= 3.4028234663852886e38; }

float read_float(const JValue& doc, const char* name, float dflt) {
    const JValue* v = doc.member(name);
    return (v && float_number(*v)) ? float(v->num) : dflt;
}

void read_float3(const JValue& doc, const char* name, const float dflt[3], float out[3]) {
    const JValue* v = doc.member(name);
    if (v && v->kind == JValue::kArray && v->items.size() >= 3 && float_number(v->items[0]) &&
        float_number(v->items[1]) && float_number(v->items[2])) {
        for (int i = 0; i < 3; ++i) out[i] = float(v->items[i].num);
    } else {
        for (int i = 0; i < 3; ++i) out[i] = dflt[i];
    }
}

bool read_bool(const JValue& doc, const char* name, bool dflt) {
    const JValue* v = doc.member(name);
    return (v && v->kind == JValue::kBool) ? v->b : dflt;
}

bool equals_ignore_case(const std::string& a, const char* b) {
    const size_t n = std::strlen(b);
    if (a.size() != n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower(static_cast<unsigned char>(a[i])) != std::tolower(static_cast<unsigned char>(b[i])))
            return false;
    return true;
}

// The importer's scalar attributes and defaults (ImportMaterial.cpp:17-52), in SelMaterial's fields;
// "displacement" has no field here and is not read.
struct Scalar {
    const char* name;
    float dflt;
    float SelMaterial::*field;
};
const Scalar kScalars[] = {
    {"metallic", 0.3f, &SelMaterial::metallic},         {"specularTint", 0.0f, &SelMaterial::specularTint},
    {"roughness", 0.5f, &SelMaterial::roughness},       {"anisotropic", 0.0f, &SelMaterial::anisotropic},
    {"sheen", 0.0f, &SelMaterial::sheen},               {"sheenTint", 0.0f, &SelMaterial::sheenTint},
    {"clearcoat", 0.0f, &SelMaterial::clearcoat},       {"clearcoatGloss", 0.0f, &SelMaterial::clearcoatGloss},
    {"specTrans", 0.0f, &SelMaterial::specTrans},       {"diffTrans", 0.0f, &SelMaterial::diffuseTrans},
    {"flatness", 0.0f, &SelMaterial::flatness},         {"ior", 1.5f, &SelMaterial::ior},
    {"scatterDistance", 0.0f, &SelMaterial::scatterDistance},
};

// DetermineShaderType (BuildModel.cpp:22-37): a case-insensitive match of the shader name, DisneySolid otherwise.
int32_t shader_of(const std::string& name) {
    static const char* const names[] = {"DisneyThin", "DisneySolid", "DeltaTransparent"};
    int32_t shader = SEL_SHADER_DISNEY_SOLID;
    for (int32_t k = 0; k < 3; ++k)
        if (equals_ignore_case(name, names[k])) shader = k;
    return shader;
}

void copy_text(const std::string& s, char* out, unsigned int capacity) {
    if (!out || capacity == 0) return;
    const size_t n = std::min<size_t>(s.size(), capacity - 1);
    std::memcpy(out, s.data(), n);
    out[n] = '\0';
}

bool parse_document(const char* json, JValue& doc) {
    std::string error;
    JReader reader(json);
    if (!reader.parse(doc, error)) {
        fail(SEL_ERR_INVALID_ARGUMENT, "malformed JSON: " + error);
        return false;
    }
    if (doc.kind != JValue::kObject) {
        fail(SEL_ERR_INVALID_ARGUMENT, "the JSON document is not an object");
        return false;
    }
    return true;
}

// Json::ReadMatrix4x4 (UtilityLib/JsonUtilities.cpp:207-252): 16 numbers, rows r0..r3 of the reference's
// row-vector matrix (translation in r3), else the identity.
void read_matrix(const JValue& doc, const char* name, float out[16]) {
    for (int k = 0; k < 16; ++k) out[k] = (k % 5 == 0) ? 1.0f : 0.0f;
    const JValue* v = doc.member(name);
    if (!v || v->kind != JValue::kArray || v->items.size() != 16) return;
    for (const JValue& x : v->items)
        if (!float_number(x)) return;
    for (int k = 0; k < 16; ++k) out[k] = float(v->items[size_t(k)].num);
}

// Json::ReadFixedString: the string when the member is one, else "".
std::string read_string(const JValue& doc, const char* name) {
    const JValue* v = doc.member(name);
    return (v && v->kind == JValue::kString) ? v->str : std::string();
}

// The "instances" (key "model") or "scenes" (key "scene") array of a scene file.
int read_instances(const JValue& doc, const char* array, const char* key, SelSceneInstance* out,
                   unsigned int capacity, unsigned int& count) {
    count = 0;
    const JValue* list = doc.member(array);
    if (!list) return SEL_OK;
    if (list->kind != JValue::kArray) return fail(SEL_ERR_INVALID_ARGUMENT, std::string(array) + " is not an array");
    for (const JValue& item : list->items) {
        if (item.kind != JValue::kObject)
            return fail(SEL_ERR_INVALID_ARGUMENT, std::string(array) + " holds a non-object");
        if (count < capacity) {
            SelSceneInstance& inst = out[count];
            std::memset(&inst, 0, sizeof(inst));
            copy_text(read_string(item, key), inst.asset, sizeof(inst.asset));
            read_matrix(item, "transform", inst.localToWorld);
        }
        ++count;
    }
    return SEL_OK;
}

}  // namespace
}  // namespace sel

using namespace sel;

extern "C" {

int sel_material_from_json(const char* json, SelMaterial* out, char* base_color_texture, unsigned int texture_capacity) {
    if (!json || !out) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    JValue doc;
    if (!parse_document(json, doc)) return SEL_ERR_INVALID_ARGUMENT;
    SelMaterial m;
    std::memset(&m, 0, sizeof(m));
    const JValue* shader = doc.member("shaderName");
    m.shader = shader && shader->kind == JValue::kString ? shader_of(shader->str) : SEL_SHADER_DISNEY_SOLID;
    const float grey[3] = {0.6f, 0.6f, 0.6f}, zero[3] = {0.0f, 0.0f, 0.0f};
    std::string texture;
    const JValue* base = doc.member("baseColor");
    if (base && base->kind == JValue::kString) {
        texture = base->str;  // a texture name: the constant colour stays 0.6 grey
        for (int i = 0; i < 3; ++i) m.baseColor[i] = grey[i];
    } else {
        read_float3(doc, "baseColor", grey, m.baseColor);
    }
    read_float3(doc, "transmittanceColor", zero, m.transmittanceColor);
    for (const Scalar& a : kScalars) m.*(a.field) = read_float(doc, a.name, a.dflt);  // a texture name: the default
    m.usesPtex = read_bool(doc, "usesPtex", false) ? 1u : 0u;
    copy_text(texture, base_color_texture, texture_capacity);
    *out = m;
    return SEL_OK;
}

int sel_disney_materials_from_json(const char* json, SelNamedMaterial* out, unsigned int capacity,
                                   unsigned int* count) {
    if (!json || !count || (capacity > 0 && !out)) return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    JValue doc;
    if (!parse_document(json, doc)) return SEL_ERR_INVALID_ARGUMENT;
    std::vector<SelNamedMaterial> all;
    for (const auto& entry : doc.members) {
        const JValue& e = entry.second;
        if (e.kind != JValue::kObject) return fail(SEL_ERR_INVALID_ARGUMENT, "material '" + entry.first + "' is not an object");
        SelNamedMaterial nm;
        std::memset(&nm, 0, sizeof(nm));
        SelMaterial& m = nm.material;
        const float one[3] = {1.0f, 1.0f, 1.0f};
        read_float3(e, "baseColor", one, m.baseColor);
        for (int i = 0; i < 3; ++i) m.transmittanceColor[i] = 1.0f;
        for (const Scalar& a : kScalars) m.*(a.field) = read_float(e, a.name, a.dflt);
        const JValue* type = e.member("type");
        m.shader = (type && type->kind == JValue::kString && type->str == "solid") ? SEL_SHADER_DISNEY_SOLID
                                                                                 : SEL_SHADER_DISNEY_THIN;
        if (const JValue* map = e.member("colorMap")) {
            if (map->kind != JValue::kString)
                return fail(SEL_ERR_INVALID_ARGUMENT, "colorMap of material '" + entry.first + "' is not a string");
            std::string path = map->str;
            for (char& c : path)
                if (c == '\\') c = '/';  // AssetFileUtils::IndependentPathSeperators
            copy_text(path, nm.colorMap, sizeof(nm.colorMap));
            m.usesPtex = path.empty() ? 0u : 1u;
        }
        copy_text(entry.first, nm.name, sizeof(nm.name));
        all.push_back(nm);
        // the same material again under each assignment name (so curves can find theirs)
        if (const JValue* assignment = e.member("assignment")) {
            if (assignment->kind != JValue::kArray)
                return fail(SEL_ERR_INVALID_ARGUMENT, "assignment of material '" + entry.first + "' is not an array");
            for (const JValue& a : assignment->items) {
                if (a.kind != JValue::kString)
                    return fail(SEL_ERR_INVALID_ARGUMENT, "assignment of material '" + entry.first + "' holds a non-string");
                SelNamedMaterial alias = nm;
                copy_text(a.str, alias.name, sizeof(alias.name));
                all.push_back(alias);
            }
        }
    }
    *count = unsigned(all.size());
    for (size_t k = 0; k < all.size() && k < capacity; ++k) out[k] = all[k];
    return SEL_OK;
}

int sel_scene_description_from_json(const char* json, SelSceneDescription* out, SelSceneInstance* models,
                                    unsigned int model_capacity, SelSceneInstance* scenes, unsigned int scene_capacity) {
    if (!json || !out || (model_capacity > 0 && !models) || (scene_capacity > 0 && !scenes))
        return fail(SEL_ERR_INVALID_ARGUMENT, "null argument");
    JValue doc;
    if (!parse_document(json, doc)) return SEL_ERR_INVALID_ARGUMENT;
    SelSceneDescription d;
    std::memset(&d, 0, sizeof(d));
    if (int rc = read_instances(doc, "instances", "model", models, model_capacity, d.modelCount)) return rc;
    if (int rc = read_instances(doc, "scenes", "scene", scenes, scene_capacity, d.sceneCount)) return rc;
    const float one[3] = {1.0f, 1.0f, 1.0f};
    read_float3(doc, "backgroundIntensity", one, d.backgroundIntensity);
    copy_text(read_string(doc, "ibl"), d.ibl, sizeof(d.ibl));
    *out = d;
    return SEL_OK;
}

}  // extern "C"
