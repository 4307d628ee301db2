// MaterialX documents whose surface shader is a standard_surface node with constant inputs, turned
// into the built-in material's properties (declarations and provenance in
// include/aurora_gb300_loaders.hpp).  The XML reader handles what MaterialX documents use:
// elements, attributes, self-closing tags, comments, the XML declaration and the five predefined
// entities.
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>

#include "../../include/aurora_gb300_loaders.hpp"

namespace agb_aurora
{
namespace
{

struct XmlElement
{
    std::string name;
    std::map<std::string, std::string> attrs;
    std::vector<std::unique_ptr<XmlElement>> children;
    std::string attr(const std::string& k) const
    {
        auto it = attrs.find(k);
        return it == attrs.end() ? std::string() : it->second;
    }
    bool has(const std::string& k) const { return attrs.count(k) != 0; }
};

class XmlReader
{
public:
    explicit XmlReader(const std::string& text) : s_(text) {}
    bool parse(XmlElement& root, std::string& error)
    {
        skipMisc();
        if (!element(root, 0))
        {
            error = "MaterialX document: " + error_ + " near byte " + std::to_string(p_);
            return false;
        }
        skipMisc();
        if (p_ != s_.size())
        {
            error = "MaterialX document: text after the root element";
            return false;
        }
        return true;
    }

private:
    const std::string& s_;
    size_t p_ = 0;
    std::string error_;

    bool fail(const std::string& what)
    {
        error_ = what;
        return false;
    }
    bool starts(const char* t) const { return s_.compare(p_, std::strlen(t), t) == 0; }
    void ws()
    {
        while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\n' || s_[p_] == '\r'))
            p_++;
    }
    // Whitespace, comments, processing instructions and a DOCTYPE between elements.
    void skipMisc()
    {
        for (;;)
        {
            ws();
            if (starts("<!--"))
            {
                size_t e = s_.find("-->", p_ + 4);
                p_       = e == std::string::npos ? s_.size() : e + 3;
            }
            else if (starts("<?") || starts("<!"))
            {
                size_t e = s_.find('>', p_);
                p_       = e == std::string::npos ? s_.size() : e + 1;
            }
            else
                return;
        }
    }
    static bool nameChar(char c)
    {
        return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_' ||
            c == ':' || c == '-' || c == '.';
    }
    std::string name()
    {
        size_t b = p_;
        while (p_ < s_.size() && nameChar(s_[p_]))
            p_++;
        return s_.substr(b, p_ - b);
    }
    static std::string unescape(const std::string& v)
    {
        std::string out;
        for (size_t i = 0; i < v.size(); i++)
        {
            if (v[i] != '&')
            {
                out += v[i];
                continue;
            }
            static const struct
            {
                const char* ent;
                char c;
            } kEnt[] = { { "&lt;", '<' }, { "&gt;", '>' }, { "&amp;", '&' }, { "&quot;", '"' }, { "&apos;", '\'' } };
            bool done = false;
            for (auto& e : kEnt)
                if (v.compare(i, std::strlen(e.ent), e.ent) == 0)
                {
                    out += e.c;
                    i += std::strlen(e.ent) - 1;
                    done = true;
                    break;
                }
            if (!done)
                out += '&';
        }
        return out;
    }
    bool element(XmlElement& el, int depth)
    {
        if (depth > 64)
            return fail("elements nested too deeply");
        if (p_ >= s_.size() || s_[p_] != '<')
            return fail("expected an element");
        p_++;
        el.name = name();
        if (el.name.empty())
            return fail("element without a name");
        for (;;)
        {
            ws();
            if (p_ >= s_.size())
                return fail("unterminated start tag");
            if (starts("/>"))
            {
                p_ += 2;
                return true;
            }
            if (s_[p_] == '>')
            {
                p_++;
                break;
            }
            std::string key = name();
            if (key.empty())
                return fail("bad attribute");
            ws();
            if (p_ >= s_.size() || s_[p_] != '=')
                return fail("attribute without a value");
            p_++;
            ws();
            if (p_ >= s_.size() || (s_[p_] != '"' && s_[p_] != '\''))
                return fail("unquoted attribute value");
            char q   = s_[p_++];
            size_t e = s_.find(q, p_);
            if (e == std::string::npos)
                return fail("unterminated attribute value");
            el.attrs[key] = unescape(s_.substr(p_, e - p_));
            p_            = e + 1;
        }
        // Content: child elements (text is ignored).
        for (;;)
        {
            skipMisc();
            if (p_ >= s_.size())
                return fail("unterminated element " + el.name);
            if (starts("</"))
            {
                p_ += 2;
                std::string closing = name();
                ws();
                if (closing != el.name || p_ >= s_.size() || s_[p_] != '>')
                    return fail("mismatched end tag for " + el.name);
                p_++;
                return true;
            }
            if (s_[p_] == '<')
            {
                el.children.push_back(std::make_unique<XmlElement>());
                if (!element(*el.children.back(), depth + 1))
                    return false;
            }
            else
                p_++; // character data
        }
    }
};

std::vector<float> numbers(const std::string& v)
{
    std::vector<float> out;
    const char* p = v.c_str();
    for (;;)
    {
        while (*p == ' ' || *p == ',' || *p == '\t')
            p++;
        if (!*p)
            break;
        char* end = nullptr;
        float f   = std::strtof(p, &end);
        if (end == p)
            return {};
        out.push_back(f);
        p = end;
    }
    return out;
}

const XmlElement* findChild(const XmlElement& root, const std::string& elementName, const std::string& nodeName)
{
    for (auto& c : root.children)
        if (c->name == elementName && (nodeName.empty() || c->attr("name") == nodeName))
            return c.get();
    return nullptr;
}

// The texture slots a standard_surface input can take from an image node (MaterialBase.cpp:91-95).
const char* textureSlot(const std::string& input)
{
    if (input == "base_color")
        return "base_color_image";
    if (input == "specular_roughness")
        return "specular_roughness_image";
    if (input == "emission_color")
        return "emission_color_image";
    if (input == "opacity")
        return "opacity_image";
    return nullptr;
}

const XmlElement* findNamed(const XmlElement& scope, const std::string& name)
{
    for (auto& c : scope.children)
        if (c->attr("name") == name)
            return c.get();
    return nullptr;
}

// The image or tiledimage node an input is connected to: directly (nodename) or through a node
// graph's output; null otherwise.
const XmlElement* connectedImage(const XmlElement& root, const XmlElement& in)
{
    const XmlElement* node = nullptr;
    if (in.has("nodegraph"))
    {
        const XmlElement* graph = findNamed(root, in.attr("nodegraph"));
        if (!graph)
            return nullptr;
        const XmlElement* out = nullptr;
        for (auto& c : graph->children)
            if (c->name == "output" && (!in.has("output") || c->attr("name") == in.attr("output")))
            {
                out = c.get();
                break;
            }
        if (!out || !out->has("nodename"))
            return nullptr;
        node = findNamed(*graph, out->attr("nodename"));
    }
    else if (in.has("nodename"))
        node = findNamed(root, in.attr("nodename"));
    return node && (node->name == "image" || node->name == "tiledimage") ? node : nullptr;
}

} // namespace

bool materialXToProperties(const std::string& document, Properties& properties, std::string& warnings)
{
    std::vector<MaterialXImage> images;
    bool ok = materialXToProperties(document, "", properties, warnings, images);
    if (!images.empty())
        warnings += "MaterialX image files are not loaded without a scene\n";
    return ok;
}

bool materialXToProperties(const std::string& document, const std::string& baseDirectory,
    Properties& properties, std::string& warnings, std::vector<MaterialXImage>& images)
{
    XmlElement root;
    std::string error;
    if (!XmlReader(document).parse(root, error))
    {
        warnings += error + "\n";
        return false;
    }
    if (root.name != "materialx")
    {
        warnings += "MaterialX document: the root element is <" + root.name + ">, not <materialx>\n";
        return false;
    }
    // The surface shader of the first surfacematerial, else the first standard_surface.
    const XmlElement* shader = nullptr;
    if (const XmlElement* mat = findChild(root, "surfacematerial", ""))
    {
        for (auto& in : mat->children)
            if (in->name == "input" && in->attr("name") == "surfaceshader")
            {
                std::string node = in->attr("nodename");
                for (auto& c : root.children)
                    if (c->attr("name") == node && c->name != "surfacematerial")
                        shader = c.get();
                if (!shader)
                {
                    warnings += "MaterialX document: surface shader '" + node + "' not found\n";
                    return false;
                }
            }
    }
    if (!shader)
        shader = findChild(root, "standard_surface", "");
    if (!shader)
    {
        warnings += "MaterialX document: no surface shader\n";
        return false;
    }
    if (shader->name != "standard_surface")
    {
        warnings += "MaterialX document: surface shader <" + shader->name +
            "> is not supported (only standard_surface)\n";
        return false;
    }
    const std::string docSpace = root.has("colorspace") ? root.attr("colorspace") : "lin_rec709";
    for (auto& in : shader->children)
    {
        if (in->name != "input")
            continue;
        const std::string n = in->attr("name"), type = in->attr("type");
        if (in->has("nodename") || in->has("nodegraph") || in->has("output") || in->has("interfacename"))
        {
            // An image (or tiledimage) node feeding a texturable input becomes that input's
            // texture: the file (sRGB-decoded when its colour space is srgb_texture), with a
            // tiledimage's uvtiling / uvoffset as the texture scale / offset.
            const XmlElement* img = connectedImage(root, *in);
            const char* slot      = textureSlot(n);
            const XmlElement* file = nullptr;
            if (img)
                for (auto& c : img->children)
                    if (c->name == "input" && c->attr("name") == "file" && c->has("value"))
                        file = c.get();
            if (slot && file)
            {
                std::string path = file->attr("value");
                if (!path.empty() && path[0] != '/' && !baseDirectory.empty())
                    path = baseDirectory + path;
                const std::string space = file->has("colorspace") ? file->attr("colorspace")
                    : img->has("colorspace")                       ? img->attr("colorspace")
                                                                   : docSpace;
                const bool linearize = space == "srgb_texture";
                const Path image     = "MaterialXImage/" + path + ":linearize:" + (linearize ? "1" : "0");
                images.push_back(MaterialXImage{ slot, image, path, linearize });
                properties[slot] = image;
                for (auto& c : img->children)
                {
                    if (c->name != "input" || !c->has("value"))
                        continue;
                    std::vector<float> f = numbers(c->attr("value"));
                    if (c->attr("name") == "uvtiling" && f.size() == 2)
                        properties[std::string(slot) + "_scale"] = vec2{ f[0], f[1] };
                    else if (c->attr("name") == "uvoffset" && f.size() == 2)
                        properties[std::string(slot) + "_offset"] = vec2{ f[0], f[1] };
                }
                continue;
            }
            warnings += "MaterialX input '" + n + "' is connected to a node graph, which is not supported; " +
                "its default is used\n";
            continue;
        }
        if (!in->has("value"))
            continue;
        const std::string v = in->attr("value");
        if (in->has("colorspace") && in->attr("colorspace") != docSpace)
            warnings += "MaterialX input '" + n + "': colour space " + in->attr("colorspace") +
                " is taken as " + docSpace + "\n";
        std::vector<float> f = numbers(v);
        if (type == "boolean")
            properties[n] = v == "true" || v == "1";
        else if (type == "integer" && f.size() == 1)
            properties[n] = int(f[0]);
        else if (type == "float" && f.size() == 1)
            properties[n] = f[0];
        else if ((type == "color3" || type == "vector3") && f.size() == 3)
            properties[n] = vec3{ f[0], f[1], f[2] };
        else if (type == "color4" && f.size() == 4)
            properties[n] = vec3{ f[0], f[1], f[2] };
        else
            warnings += "MaterialX input '" + n + "' of type " + type + " (value '" + v + "') is not supported\n";
    }
    return true;
}

bool materialXFileToProperties(const std::string& path, Properties& properties, std::string& warnings,
    std::vector<MaterialXImage>* images)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
    {
        warnings += "cannot read MaterialX file " + path + "\n";
        return false;
    }
    std::ostringstream s;
    s << f.rdbuf();
    // Image files are found beside the document (the reference prefixes relative texture paths
    // with the document's folder, glTFLoader.cpp:310-327).
    size_t k = path.find_last_of("/\\");
    std::string dir = k == std::string::npos ? std::string() : path.substr(0, k + 1);
    std::vector<MaterialXImage> local;
    bool ok = materialXToProperties(s.str(), dir, properties, warnings, images ? *images : local);
    if (!images && !local.empty())
        warnings += "MaterialX image files are not loaded without a scene\n";
    return ok;
}

} // namespace agb_aurora
