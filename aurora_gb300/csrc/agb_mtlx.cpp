// MaterialX documents whose surface shader is a standard_surface node with constant inputs, turned
// into the built-in material's properties (declarations and provenance in
// include/aurora_gb300_loaders.hpp).  The XML reader handles what MaterialX documents use:
// elements, attributes, self-closing tags, comments, the XML declaration and the five predefined
// entities.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>

#include "../../include/agb.h"
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

// ------------------------------------------------------------------------------ node graphs
// A standard_surface input connected to a node graph is compiled into a program of the
// operations agb_material_graphs_set runs per hit (include/agb.h); the reference generates
// shader code for the same graph (MaterialX/BSDFCodeGenerator.cpp).  Nodes are compiled on demand
// from the input back to the graph's sources, once each per scope; custom nodes (a nodedef with
// a nodegraph implementing it in the same document) are expanded with their interface inputs
// bound to the node's inputs.  The program travels as the material property `materialx_graph`,
// a list of strings: "op <code> <dst> <a> <b> <c> <d> <imm>", "const <x> <y> <z> <w>" (in
// constant order) and "image <image path>" (in image order, the IMAGE operand).
class GraphCompiler
{
public:
    struct Value
    {
        int reg = -1;
        int n   = 0; // components (1 to 4)
    };

    GraphCompiler(const XmlElement& root, const std::string& baseDirectory, const std::string& docSpace,
        std::string& warnings, std::vector<MaterialXImage>& images) :
        root_(root), base_(baseDirectory), space_(docSpace), warnings_(warnings), images_(images)
    {
    }

    // Compiles the shader input `in` and writes it to material field `field` (AGB_GOUT_*) of `n`
    // components; false (nothing emitted) when some node on the way is not supported.
    bool compileOutput(const XmlElement& in, int field, int n)
    {
        const size_t opMark = ops_.size(), kMark = consts_.size(), imMark = imagePaths_.size();
        const int regMark = nextReg_;
        auto cacheMark    = cache_;
        std::string why;
        Value v;
        if (resolveInput(in, Scope{ &root_, nullptr, nullptr }, v, why))
        {
            if (v.n == 1 && n > 1)
                v = splat(v);
            if (v.reg >= 0 && !error_)
            {
                emit(AGB_GOP_OUTPUT, 0, v.reg, 0, 0, 0, uint16_t(field));
                return true;
            }
        }
        // Roll back what this input emitted.
        ops_.resize(opMark);
        consts_.resize(kMark);
        imagePaths_.resize(imMark);
        nextReg_ = regMark;
        cache_   = cacheMark;
        error_   = false;
        warnings_ += "MaterialX input '" + in.attr("name") + "': " + (why.empty() ? "the node graph is too large" : why) +
            "; its default is used\n";
        return false;
    }

    bool empty() const { return ops_.empty(); }

    // The program with virtual registers mapped onto the AGB_GRAPH_REGS registers: a register is
    // free again after the last operation that reads it (operands are read before the result is
    // written, so a result may take an operand's register).  False when more are live at once.
    bool program(Strings& out)
    {
        std::vector<int> lastUse(size_t(nextReg_), -1);
        for (size_t k = 0; k < ops_.size(); k++)
            for (int q = 0; q < operands(ops_[k].op); q++)
                lastUse[size_t((&ops_[k].a)[q])] = int(k);
        std::vector<int> phys(size_t(nextReg_), -1);
        std::vector<int> freeRegs;
        for (int r = AGB_GRAPH_REGS - 1; r >= 0; r--)
            freeRegs.push_back(r);
        std::vector<agb_graph_op> mapped;
        for (size_t k = 0; k < ops_.size(); k++)
        {
            const VOp& v = ops_[k];
            agb_graph_op o{};
            o.op  = uint8_t(v.op);
            o.imm = v.imm;
            int in[4] = { 0, 0, 0, 0 };
            for (int q = 0; q < operands(v.op); q++)
                in[q] = phys[size_t((&v.a)[q])];
            o.a = uint8_t(in[0]);
            o.b = uint8_t(in[1]);
            o.c = uint8_t(in[2]);
            o.d = uint8_t(v.op == AGB_GOP_DOT || v.op == AGB_GOP_NORMALIZE || v.op == AGB_GOP_LENGTH ? v.d : in[3]);
            // Operands read for the last time release their registers before the result takes one.
            for (int q = 0; q < operands(v.op); q++)
            {
                const int vr = (&v.a)[q];
                if (lastUse[size_t(vr)] == int(k) && phys[size_t(vr)] >= 0)
                {
                    freeRegs.push_back(phys[size_t(vr)]);
                    phys[size_t(vr)] = -1;
                }
            }
            if (v.op != AGB_GOP_OUTPUT)
            {
                if (freeRegs.empty())
                    return false;
                phys[size_t(v.dst)] = freeRegs.back();
                freeRegs.pop_back();
                o.dst = uint8_t(phys[size_t(v.dst)]);
                if (lastUse[size_t(v.dst)] < 0) // never read
                {
                    freeRegs.push_back(phys[size_t(v.dst)]);
                    phys[size_t(v.dst)] = -1;
                }
            }
            mapped.push_back(o);
        }
        char buf[160];
        for (const agb_graph_op& o : mapped)
        {
            std::snprintf(buf, sizeof buf, "op %d %d %d %d %d %d %d", o.op, o.dst, o.a, o.b, o.c, o.d, o.imm);
            out.push_back(buf);
        }
        for (size_t k = 0; k + 3 < consts_.size(); k += 4)
        {
            std::snprintf(buf, sizeof buf, "const %.9g %.9g %.9g %.9g", consts_[k], consts_[k + 1], consts_[k + 2],
                consts_[k + 3]);
            out.push_back(buf);
        }
        for (const std::string& p : imagePaths_)
            out.push_back("image " + p);
        return true;
    }

private:
    struct Scope
    {
        const XmlElement* graph;  // the element whose children are the nodes (the document or a nodegraph)
        const XmlElement* call;   // the custom node a nodedef's graph implements, or null
        const Scope* parent;
    };

    const XmlElement& root_;
    std::string base_, space_;
    std::string& warnings_;
    std::vector<MaterialXImage>& images_;
    // Operations over virtual registers (one per value), mapped onto registers by program().
    struct VOp
    {
        int op, a, b, c, d, dst; // a .. d contiguous: the operands
        uint16_t imm;
    };
    std::vector<VOp> ops_;
    std::vector<float> consts_;
    std::vector<std::string> imagePaths_;
    std::map<std::string, Value> cache_;
    int nextReg_ = 0;
    bool error_  = false;
    int depth_   = 0;

    // Register operands each operation reads (a, b, c, d in order).
    static int operands(int op)
    {
        switch (op)
        {
        case AGB_GOP_CONST:
        case AGB_GOP_INPUT: return 0;
        case AGB_GOP_ADD:
        case AGB_GOP_SUB:
        case AGB_GOP_MUL:
        case AGB_GOP_DIV:
        case AGB_GOP_MIN:
        case AGB_GOP_MAX:
        case AGB_GOP_POW:
        case AGB_GOP_MOD:
        case AGB_GOP_DOT:
        case AGB_GOP_NORMALMAP: return 2;
        case AGB_GOP_CLAMP:
        case AGB_GOP_MIX: return 3;
        case AGB_GOP_COMBINE:
        case AGB_GOP_SELECT: return 4;
        default: return 1;
        }
    }
    int reg()
    {
        if (nextReg_ >= AGB_GRAPH_MAX_OPS)
        {
            error_ = true;
            return 0;
        }
        return nextReg_++;
    }
    void emit(int op, int dst, int a, int b, int c, int d, uint16_t imm)
    {
        ops_.push_back(VOp{ op, a, b, c, d, dst, imm });
        if (ops_.size() > AGB_GRAPH_MAX_OPS)
            error_ = true;
    }
    Value op1(int op, Value a, int n = -1, uint16_t imm = 0)
    {
        Value r{ reg(), n < 0 ? a.n : n };
        emit(op, r.reg, a.reg, 0, 0, 0, imm);
        return r;
    }
    Value splat(Value a)
    {
        Value r = op1(AGB_GOP_SWIZZLE, a, 4, 0);
        return r;
    }
    // Operands of a component-wise operation: a scalar meets a vector as its splat.
    void widen(Value& a, Value& b)
    {
        if (a.n == 1 && b.n > 1)
            a = Value{ splat(a).reg, b.n };
        else if (b.n == 1 && a.n > 1)
            b = Value{ splat(b).reg, a.n };
    }
    Value op2(int op, Value a, Value b)
    {
        widen(a, b);
        Value r{ reg(), std::max(a.n, b.n) };
        emit(op, r.reg, a.reg, b.reg, 0, 0, 0);
        return r;
    }
    Value constant(const std::vector<float>& f, int n)
    {
        if (consts_.size() / 4 >= 65536)
        {
            error_ = true;
            return Value{ 0, n };
        }
        const uint16_t k = uint16_t(consts_.size() / 4);
        for (int c = 0; c < 4; c++)
            consts_.push_back(c < int(f.size()) ? f[c] : (f.size() == 1 ? f[0] : 0.f));
        Value r{ reg(), n };
        emit(AGB_GOP_CONST, r.reg, 0, 0, 0, 0, k);
        return r;
    }
    static int components(const std::string& type)
    {
        if (type == "float" || type == "integer" || type == "boolean")
            return 1;
        if (type == "vector2")
            return 2;
        if (type == "vector3" || type == "color3")
            return 3;
        if (type == "vector4" || type == "color4")
            return 4;
        return 0;
    }
    Value valueOf(const std::string& type, const std::string& text, std::string& why)
    {
        const int n = components(type);
        if (!n)
        {
            why = "value of type " + type + " is not supported";
            return Value{};
        }
        std::vector<float> f;
        if (type == "boolean")
            f.push_back(text == "true" || text == "1" ? 1.f : 0.f);
        else
            f = numbers(text);
        if (int(f.size()) != n)
        {
            why = "value '" + text + "' is not a " + type;
            return Value{};
        }
        return constant(f, n);
    }

    const XmlElement* childInput(const XmlElement& node, const std::string& name) const
    {
        for (auto& c : node.children)
            if (c->name == "input" && c->attr("name") == name)
                return c.get();
        return nullptr;
    }
    // An image file sampled at uv (an image node's file input; its colour space decides the sRGB
    // decode, filtertype "closest" nearest sampling): the IMAGE operation on the graph's image list.
    Value sampleFile(const XmlElement& node, const XmlElement& file, Value uv, int n)
    {
        std::string path = file.attr("value");
        if (!path.empty() && path[0] != '/' && !base_.empty())
            path = base_ + path;
        const std::string sp = file.has("colorspace") ? file.attr("colorspace")
            : node.has("colorspace")                       ? node.attr("colorspace")
                                                           : space_;
        const bool linearize  = sp == "srgb_texture";
        const XmlElement* ft  = childInput(node, "filtertype");
        const bool nearest    = ft && ft->attr("value") == "closest";
        const std::string img = "MaterialXImage/" + path + ":linearize:" + (linearize ? "1" : "0");
        int index             = -1;
        for (size_t q = 0; q < imagePaths_.size(); q++)
            if (imagePaths_[q] == img + (nearest ? ":nearest" : ""))
                index = int(q);
        if (index < 0)
        {
            index = int(imagePaths_.size());
            imagePaths_.push_back(img + (nearest ? ":nearest" : ""));
            images_.push_back(MaterialXImage{ "materialx_graph", img, path, linearize });
        }
        Value out{ reg(), std::min(n, 4) };
        emit(AGB_GOP_IMAGE, out.reg, uv.reg, 0, 0, 0, uint16_t(index));
        return out;
    }
    const XmlElement* nodedefFor(const std::string& category) const
    {
        for (auto& c : root_.children)
            if (c->name == "nodedef" && c->attr("node") == category)
                return c.get();
        return nullptr;
    }
    const XmlElement* graphImplementing(const XmlElement& nodedef) const
    {
        for (auto& c : root_.children)
            if (c->name == "nodegraph" && c->attr("nodedef") == nodedef.attr("name"))
                return c.get();
        return nullptr;
    }
    static const XmlElement* outputOf(const XmlElement& graph, const std::string& name)
    {
        for (auto& c : graph.children)
            if (c->name == "output" && (name.empty() || c->attr("name") == name))
                return c.get();
        return nullptr;
    }

    // The value an <input> (or a graph <output>) element supplies in scope S.
    bool resolveInput(const XmlElement& in, const Scope& S, Value& out, std::string& why)
    {
        if (++depth_ > 64)
        {
            depth_--;
            why = "the node graph is nested too deeply";
            return false;
        }
        bool ok = resolveInputAt(in, S, out, why);
        depth_--;
        return ok && !error_;
    }
    bool resolveInputAt(const XmlElement& in, const Scope& S, Value& out, std::string& why)
    {
        if (in.has("nodename"))
        {
            const XmlElement* node = findNamed(*S.graph, in.attr("nodename"));
            if (!node)
            {
                why = "node '" + in.attr("nodename") + "' not found";
                return false;
            }
            return compileNode(*node, S, in.attr("output"), out, why);
        }
        if (in.has("nodegraph"))
        {
            const XmlElement* graph = findNamed(root_, in.attr("nodegraph"));
            const XmlElement* o     = graph ? outputOf(*graph, in.attr("output")) : nullptr;
            if (!o)
            {
                why = "node graph output '" + in.attr("nodegraph") + "/" + in.attr("output") + "' not found";
                return false;
            }
            return resolveInput(*o, Scope{ graph, nullptr, &S }, out, why);
        }
        if (in.has("interfacename"))
        {
            const std::string name = in.attr("interfacename");
            if (S.call)
            {
                // A custom node's input, or the nodedef's default.
                if (const XmlElement* ci = childInput(*S.call, name))
                    return resolveInput(*ci, *S.parent, out, why);
                const XmlElement* def = nodedefFor(S.call->name);
                const XmlElement* di  = def ? childInput(*def, name) : nullptr;
                if (di && di->has("value"))
                {
                    out = valueOf(di->attr("type"), di->attr("value"), why);
                    return out.reg >= 0;
                }
                why = "interface input '" + name + "' has no value";
                return false;
            }
            // A node graph's own interface input.
            if (const XmlElement* gi = childInput(*S.graph, name))
                return resolveInput(*gi, S.parent ? *S.parent : S, out, why);
            why = "interface input '" + name + "' not found";
            return false;
        }
        if (in.has("value"))
        {
            out = valueOf(in.attr("type"), in.attr("value"), why);
            return out.reg >= 0;
        }
        why = "input '" + in.attr("name") + "' has no value or connection";
        return false;
    }

    // The element holding the literal value an input takes in scope S, following interface
    // bindings (a node graph's own interface input, a custom node's input or its nodedef's
    // default); null when the input is fed by a node.
    const XmlElement* literalInput(const XmlElement* in, const Scope* S) const
    {
        for (int hops = 0; in && !in->has("value") && hops < 64; hops++)
        {
            if (!in->has("interfacename") || !S)
                return nullptr;
            const std::string name = in->attr("interfacename");
            if (S->call)
            {
                if (const XmlElement* ci = childInput(*S->call, name))
                {
                    in = ci;
                    S  = S->parent;
                }
                else
                {
                    const XmlElement* def = nodedefFor(S->call->name);
                    in                    = def ? childInput(*def, name) : nullptr;
                    S                     = nullptr;
                }
            }
            else
            {
                in = childInput(*S->graph, name);
                S  = S->parent ? S->parent : S;
            }
        }
        return in && in->has("value") ? in : nullptr;
    }

    // The named input of a node, or `def` (of `type`) when it is absent.
    bool input(const XmlElement& node, const Scope& S, const char* name, const std::string& type, const char* def,
        Value& out, std::string& why)
    {
        if (const XmlElement* in = childInput(node, name))
            return resolveInput(*in, S, out, why);
        out = valueOf(type, def, why);
        return out.reg >= 0;
    }

    bool compileNode(const XmlElement& node, const Scope& S, const std::string& output, Value& out, std::string& why)
    {
        // Keyed by the node and the whole chain of custom-node expansions it sits in: the same
        // element inside a nodegraph implementation takes other inputs in another expansion.
        std::string k;
        char part[32];
        std::snprintf(part, sizeof part, "%p", static_cast<const void*>(&node));
        k += part;
        for (const Scope* q = &S; q; q = q->parent)
        {
            std::snprintf(part, sizeof part, "/%p", static_cast<const void*>(q->call));
            k += part;
        }
        k += "/" + output;
        auto it             = cache_.find(k);
        if (it != cache_.end())
        {
            out = it->second;
            return true;
        }
        bool ok = compileNodeUncached(node, S, output, out, why);
        if (ok)
            cache_[k] = out;
        return ok;
    }

    bool compileNodeUncached(const XmlElement& node, const Scope& S, const std::string& output, Value& out,
        std::string& why)
    {
        const std::string cat  = node.name;
        const std::string type = node.attr("type");
        const int n            = components(type);
        // A custom node: its nodegraph implementation with this node as the interface.
        if (const XmlElement* def = nodedefFor(cat))
        {
            const XmlElement* impl = graphImplementing(*def);
            const XmlElement* o    = impl ? outputOf(*impl, output) : nullptr;
            if (!o)
            {
                why = "node <" + cat + "> has no node graph implementation in the document";
                return false;
            }
            return resolveInput(*o, Scope{ impl, &node, &S }, out, why);
        }
        Value a, b, c, d;
        auto in = [&](const char* name, const std::string& t, const char* def, Value& v) {
            return input(node, S, name, t, def, v, why);
        };
        const std::string zero = n == 1 ? "0" : n == 2 ? "0, 0" : n == 3 ? "0, 0, 0" : "0, 0, 0, 0";
        const std::string one  = n == 1 ? "1" : n == 2 ? "1, 1" : n == 3 ? "1, 1, 1" : "1, 1, 1, 1";
        static const std::map<std::string, int> binary = { { "add", AGB_GOP_ADD }, { "subtract", AGB_GOP_SUB },
            { "multiply", AGB_GOP_MUL }, { "divide", AGB_GOP_DIV }, { "modulo", AGB_GOP_MOD },
            { "power", AGB_GOP_POW }, { "min", AGB_GOP_MIN }, { "max", AGB_GOP_MAX } };
        static const std::map<std::string, int> unary = { { "floor", AGB_GOP_FLOOR }, { "ceil", AGB_GOP_CEIL },
            { "absval", AGB_GOP_ABS }, { "sin", AGB_GOP_SIN }, { "cos", AGB_GOP_COS }, { "sqrt", AGB_GOP_SQRT },
            { "sign", AGB_GOP_SIGN } };
        if (!n && cat != "extract")
        {
            why = "node <" + cat + "> of type " + type + " is not supported";
            return false;
        }
        if (cat == "constant")
            return in("value", type, zero.c_str(), out);
        if (cat == "dot") // the pass-through node
            return in("in", type, zero.c_str(), out);
        if (binary.count(cat))
        {
            const bool unitB = cat == "multiply" || cat == "divide" || cat == "modulo" || cat == "power";
            if (!in("in1", type, zero.c_str(), a))
                return false;
            const XmlElement* i2 = childInput(node, "in2");
            // A second operand of float type on a vector node (the MaterialX "FA" forms).
            const std::string t2 = i2 && i2->has("type") ? i2->attr("type") : type;
            if (!in("in2", t2, unitB ? (components(t2) == 1 ? "1" : one.c_str()) : (components(t2) == 1 ? "0" : zero.c_str()), b))
                return false;
            out   = op2(binary.at(cat), a, b);
            out.n = n;
            return true;
        }
        if (unary.count(cat))
        {
            if (!in("in", type, zero.c_str(), a))
                return false;
            out = op1(unary.at(cat), a, n);
            return true;
        }
        if (cat == "clamp")
        {
            const XmlElement* lo = childInput(node, "low");
            const XmlElement* hi = childInput(node, "high");
            const std::string tl = lo && lo->has("type") ? lo->attr("type") : type;
            const std::string th = hi && hi->has("type") ? hi->attr("type") : type;
            if (!in("in", type, zero.c_str(), a) || !in("low", tl, components(tl) == 1 ? "0" : zero.c_str(), b) ||
                !in("high", th, components(th) == 1 ? "1" : one.c_str(), c))
                return false;
            widen(a, b);
            widen(a, c);
            out = Value{ reg(), n };
            emit(AGB_GOP_CLAMP, out.reg, a.reg, b.reg, c.reg, 0, 0);
            return true;
        }
        if (cat == "mix")
        {
            const XmlElement* m  = childInput(node, "mix");
            const std::string tm = m && m->has("type") ? m->attr("type") : "float";
            if (!in("fg", type, zero.c_str(), a) || !in("bg", type, zero.c_str(), b) ||
                !in("mix", tm, components(tm) == 1 ? "0" : zero.c_str(), c))
                return false;
            widen(a, c);
            widen(b, c);
            out = Value{ reg(), n };
            emit(AGB_GOP_MIX, out.reg, a.reg, b.reg, c.reg, 0, 0);
            return true;
        }
        if (cat == "dotproduct" || cat == "normalize" || cat == "magnitude")
        {
            const XmlElement* i1 = childInput(node, cat == "dotproduct" ? "in1" : "in");
            const std::string ti = i1 && i1->has("type") ? i1->attr("type") : "vector3";
            const int ni         = components(ti);
            if (!ni)
            {
                why = "node <" + cat + "> input type " + ti + " is not supported";
                return false;
            }
            const std::string z = ni == 2 ? "0, 0" : ni == 3 ? "0, 0, 0" : "0, 0, 0, 0";
            if (!in(cat == "dotproduct" ? "in1" : "in", ti, z.c_str(), a))
                return false;
            if (cat == "dotproduct" && !in("in2", ti, z.c_str(), b))
                return false;
            out = Value{ reg(), n };
            emit(cat == "dotproduct" ? AGB_GOP_DOT : cat == "normalize" ? AGB_GOP_NORMALIZE : AGB_GOP_LENGTH, out.reg,
                a.reg, cat == "dotproduct" ? b.reg : a.reg, 0, uint8_t(ni), 0);
            return true;
        }
        if (cat == "extract")
        {
            const XmlElement* i1 = childInput(node, "in");
            const std::string ti = i1 && i1->has("type") ? i1->attr("type") : "vector3";
            const XmlElement* ix = childInput(node, "index");
            const int index      = ix && ix->has("value") ? std::atoi(ix->attr("value").c_str()) : 0;
            if (!components(ti) || index < 0 || index >= components(ti) || (ix && !ix->has("value")))
            {
                why = "node <extract> needs a constant index within its input";
                return false;
            }
            if (!in("in", ti, "0, 0, 0", a))
                return false;
            out = op1(AGB_GOP_SWIZZLE, a, 1, uint16_t(index * 0x55));
            return true;
        }
        if (cat == "swizzle")
        {
            const XmlElement* ch = childInput(node, "channels");
            const std::string chans = ch ? ch->attr("value") : "";
            const XmlElement* i1    = childInput(node, "in");
            const std::string ti    = i1 && i1->has("type") ? i1->attr("type") : "vector3";
            if (chans.empty() || int(chans.size()) > 4 || !components(ti))
            {
                why = "node <swizzle> needs its channels";
                return false;
            }
            uint16_t imm = 0;
            for (size_t q = 0; q < 4; q++)
            {
                const char cc = chans[std::min(q, chans.size() - 1)];
                const int src = (cc == 'x' || cc == 'r') ? 0 : (cc == 'y' || cc == 'g') ? 1 : (cc == 'z' || cc == 'b') ? 2 : 3;
                imm           = uint16_t(imm | (src << (2 * q)));
            }
            if (!in("in", ti, "0, 0, 0", a))
                return false;
            out = op1(AGB_GOP_SWIZZLE, a, int(chans.size()), imm);
            return true;
        }
        if (cat == "combine2" || cat == "combine3" || cat == "combine4")
        {
            Value v[4];
            const int k = cat[7] - '0';
            for (int q = 0; q < 4; q++)
            {
                if (q < k)
                {
                    const std::string nm = "in" + std::to_string(q + 1);
                    const XmlElement* iq  = childInput(node, nm);
                    if (iq && iq->has("type") && components(iq->attr("type")) != 1)
                    {
                        why = "node <" + cat + "> with vector inputs is not supported";
                        return false;
                    }
                    if (!in(nm.c_str(), "float", "0", v[q]))
                        return false;
                }
                else
                    v[q] = v[0];
            }
            out = Value{ reg(), n };
            emit(AGB_GOP_COMBINE, out.reg, v[0].reg, v[1].reg, v[2].reg, v[3].reg, 0);
            return true;
        }
        if (cat == "ifgreater" || cat == "ifgreatereq" || cat == "ifequal")
        {
            if (!in("value1", "float", "1", a) || !in("value2", "float", "0", b) ||
                !in("in1", type, zero.c_str(), c) || !in("in2", type, zero.c_str(), d))
                return false;
            out = Value{ reg(), n };
            emit(AGB_GOP_SELECT, out.reg, a.reg, b.reg, c.reg, d.reg,
                uint16_t(cat == "ifgreater" ? 0 : cat == "ifgreatereq" ? 1 : 2));
            return true;
        }
        if (cat == "switch")
        {
            // in1 .. in10 chosen by floor(which): a chain of which >= k selections.
            Value which;
            if (!in("which", "float", "0", which) || !in("in1", type, zero.c_str(), out))
                return false;
            for (int q = 2; q <= 10; q++)
            {
                const std::string nm = "in" + std::to_string(q);
                if (!childInput(node, nm))
                    continue;
                Value vq, kq = constant({ float(q - 1) }, 1);
                if (!in(nm.c_str(), type, zero.c_str(), vq))
                    return false;
                Value r{ reg(), n };
                emit(AGB_GOP_SELECT, r.reg, which.reg, kq.reg, vq.reg, out.reg, 1);
                out = r;
            }
            return true;
        }
        if (cat == "texcoord" || cat == "position" || cat == "normal" || cat == "tangent" || cat == "bitangent")
        {
            const XmlElement* sp = childInput(node, "space");
            const std::string space = sp ? sp->attr("value") : "object";
            int which = AGB_GIN_TEXCOORD;
            if (cat == "texcoord")
            {
                const XmlElement* ix = childInput(node, "index");
                if (ix && ix->attr("value") != "0")
                    warnings_ += "MaterialX <texcoord> index " + ix->attr("value") + " is read as index 0\n";
            }
            else if (cat == "position")
                which = space == "world" ? AGB_GIN_POSITION_WORLD : AGB_GIN_POSITION_OBJECT;
            else if (cat == "normal")
                which = space == "world" ? AGB_GIN_NORMAL_WORLD : AGB_GIN_NORMAL_OBJECT;
            else
            {
                if (space != "world")
                    warnings_ += "MaterialX <" + cat + "> in " + space + " space is read in world space\n";
                which = cat == "tangent" ? AGB_GIN_TANGENT_WORLD : AGB_GIN_BITANGENT_WORLD;
            }
            out = Value{ reg(), cat == "texcoord" ? 2 : 3 };
            emit(AGB_GOP_INPUT, out.reg, 0, 0, 0, 0, uint16_t(which));
            return true;
        }
        if (cat == "image" || cat == "tiledimage")
        {
            const XmlElement* file = childInput(node, "file");
            if (!file || !file->has("value"))
            {
                why = "node <" + cat + "> has no file";
                return false;
            }
            for (const char* am : { "uaddressmode", "vaddressmode" })
                if (const XmlElement* m = childInput(node, am))
                    if (m->attr("value") != "periodic")
                        warnings_ += "MaterialX <" + cat + "> " + am + " " + m->attr("value") + " is sampled periodic\n";
            Value uv;
            if (childInput(node, "texcoord"))
            {
                if (!in("texcoord", "vector2", "0, 0", uv))
                    return false;
            }
            else
            {
                uv = Value{ reg(), 2 };
                emit(AGB_GOP_INPUT, uv.reg, 0, 0, 0, 0, AGB_GIN_TEXCOORD);
            }
            if (cat == "tiledimage")
            {
                // uv x uvtiling + uvoffset.
                Value tiling, offset;
                if (!in("uvtiling", "vector2", "1, 1", tiling) || !in("uvoffset", "vector2", "0, 0", offset))
                    return false;
                uv = op2(AGB_GOP_ADD, op2(AGB_GOP_MUL, uv, tiling), offset);
            }
            out = sampleFile(node, *file, uv, n);
            return true;
        }
        if (cat == "adsk:bitmap" || cat == "adsk:normal_map")
        {
            // Autodesk's texture nodes (their node library is not part of the reference): the file
            // at texcoord x uv_scale + uv_offset; a bitmap's value scaled by rgbamount and, with
            // invert, subtracted from 1; a normal map's tangent-space normal with its xy scaled by
            // normal_scale.  The real-world mapping (realworld_scale / realworld_offset, in
            // document distance units) and rotation_angle are not applied.
            const XmlElement* file = childInput(node, "file");
            if (!file || !file->has("value"))
            {
                why = "node <" + cat + "> has no file";
                return false;
            }
            auto constantIs = [&](const char* name, std::vector<float> want) {
                const XmlElement* c = childInput(node, name);
                return !c || (c->has("value") && numbers(c->attr("value")) == want);
            };
            if (!constantIs("realworld_scale", { 1.f, 1.f }) || !constantIs("realworld_offset", { 0.f, 0.f }) ||
                !constantIs("rotation_angle", { 0.f }))
                warnings_ += "MaterialX <" + cat + "> '" + node.attr("name") +
                    "': realworld_scale / realworld_offset / rotation_angle are not applied\n";
            Value uv{ reg(), 2 }, scale, offset;
            emit(AGB_GOP_INPUT, uv.reg, 0, 0, 0, 0, AGB_GIN_TEXCOORD);
            if (!in("uv_scale", "vector2", "1, 1", scale) || !in("uv_offset", "vector2", "0, 0", offset))
                return false;
            uv = op2(AGB_GOP_ADD, op2(AGB_GOP_MUL, uv, scale), offset);
            if (cat == "adsk:normal_map")
            {
                Value tex = sampleFile(node, *file, uv, 3);
                if (!in("normal_scale", "float", "1", b))
                    return false;
                out = Value{ reg(), 3 };
                emit(AGB_GOP_NORMALMAP, out.reg, tex.reg, b.reg, 0, 0, 0);
                return true;
            }
            out = sampleFile(node, *file, uv, n);
            if (childInput(node, "rgbamount"))
            {
                if (!in("rgbamount", "float", "1", a))
                    return false;
                out   = op2(AGB_GOP_MUL, out, a);
                out.n = std::min(n, 4);
            }
            const XmlElement* inv = childInput(node, "invert");
            if (inv && (inv->attr("value") == "true" || inv->attr("value") == "1"))
            {
                Value one = valueOf("float", "1", why);
                out       = op2(AGB_GOP_SUB, one, out);
                out.n     = std::min(n, 4);
            }
            return true;
        }
        if (cat == "normalmap")
        {
            const XmlElement* sp = childInput(node, "space");
            if (sp && sp->attr("value") != "tangent")
            {
                why = "node <normalmap> in " + sp->attr("value") + " space is not supported";
                return false;
            }
            if (!in("in", "vector3", "0.5, 0.5, 1", a) || !in("scale", "float", "1", b))
                return false;
            out = Value{ reg(), 3 };
            emit(AGB_GOP_NORMALMAP, out.reg, a.reg, b.reg, 0, 0, 0);
            return true;
        }
        if (cat == "luminance")
        {
            if (!in("in", "color3", "0, 0, 0", a) || !in("lumacoeffs", "color3", "0.2722287, 0.6740818, 0.0536895", b))
                return false;
            out = Value{ reg(), n };
            emit(AGB_GOP_DOT, out.reg, a.reg, b.reg, 0, 3, 0);
            return true;
        }
        if (cat == "invert")
        {
            const XmlElement* am = childInput(node, "amount");
            const std::string ta = am && am->has("type") ? am->attr("type") : type;
            if (!in("in", type, zero.c_str(), a) || !in("amount", ta, components(ta) == 1 ? "1" : one.c_str(), b))
                return false;
            out   = op2(AGB_GOP_SUB, b, a);
            out.n = n;
            return true;
        }
        if (cat == "remap")
        {
            // outlow + (in - inlow) (outhigh - outlow) / (inhigh - inlow)
            Value lo, hi, olo, ohi;
            if (!in("in", type, zero.c_str(), a) || !in("inlow", type, zero.c_str(), lo) ||
                !in("inhigh", type, one.c_str(), hi) || !in("outlow", type, zero.c_str(), olo) ||
                !in("outhigh", type, one.c_str(), ohi))
                return false;
            out   = op2(AGB_GOP_ADD, olo,
                  op2(AGB_GOP_DIV, op2(AGB_GOP_MUL, op2(AGB_GOP_SUB, a, lo), op2(AGB_GOP_SUB, ohi, olo)),
                      op2(AGB_GOP_SUB, hi, lo)));
            out.n = n;
            return true;
        }
        if (cat == "convert")
        {
            const XmlElement* i1 = childInput(node, "in");
            const std::string ti = i1 && i1->has("type") ? i1->attr("type") : type;
            if (!components(ti) || !in("in", ti, "0", a))
                return false;
            out = a.n == 1 && n > 1 ? Value{ splat(a).reg, n } : Value{ a.reg, n };
            return true;
        }
        if (cat == "ramplr" || cat == "ramptb")
        {
            Value uv, t, lo0, hi1;
            if (!in("valuel", type, zero.c_str(), a) || !in("valuer", type, zero.c_str(), b))
                return false;
            if (childInput(node, "texcoord"))
            {
                if (!in("texcoord", "vector2", "0, 0", uv))
                    return false;
            }
            else
            {
                uv = Value{ reg(), 2 };
                emit(AGB_GOP_INPUT, uv.reg, 0, 0, 0, 0, AGB_GIN_TEXCOORD);
            }
            t   = op1(AGB_GOP_SWIZZLE, uv, 1, uint16_t(cat == "ramplr" ? 0x00 : 0x55));
            lo0 = constant({ 0.f }, 1);
            hi1 = constant({ 1.f }, 1);
            Value tc{ reg(), 1 };
            emit(AGB_GOP_CLAMP, tc.reg, t.reg, lo0.reg, hi1.reg, 0, 0);
            if (n > 1)
                tc = Value{ splat(tc).reg, n };
            out = Value{ reg(), n };
            emit(AGB_GOP_MIX, out.reg, b.reg, a.reg, tc.reg, 0, 0);
            return true;
        }
        if (cat == "smoothstep")
        {
            // t = clamp((in - low) / (high - low), 0, 1); t^2 (3 - 2t), component-wise.
            Value lo, hi;
            if (!in("in", type, zero.c_str(), a) || !in("low", type, zero.c_str(), lo) ||
                !in("high", type, one.c_str(), hi))
                return false;
            Value t = op2(AGB_GOP_DIV, op2(AGB_GOP_SUB, a, lo), op2(AGB_GOP_SUB, hi, lo));
            Value z = valueOf("float", "0", why), u = valueOf("float", "1", why);
            Value c{ reg(), t.n };
            emit(AGB_GOP_CLAMP, c.reg, t.reg, z.reg, u.reg, 0, 0);
            Value three = valueOf("float", "3", why), two = valueOf("float", "2", why);
            out   = op2(AGB_GOP_MUL, op2(AGB_GOP_MUL, c, c), op2(AGB_GOP_SUB, three, op2(AGB_GOP_MUL, two, c)));
            out.n = n;
            return true;
        }
        if (cat == "crossproduct")
        {
            // in1.yzx in2.zxy - in1.zxy in2.yzx
            if (!in("in1", "vector3", "0, 0, 0", a) || !in("in2", "vector3", "0, 0, 0", b))
                return false;
            const uint16_t yzx = 1 | (2 << 2), zxy = 2 | (1 << 4);
            out   = op2(AGB_GOP_SUB, op2(AGB_GOP_MUL, op1(AGB_GOP_SWIZZLE, a, 3, yzx), op1(AGB_GOP_SWIZZLE, b, 3, zxy)),
                  op2(AGB_GOP_MUL, op1(AGB_GOP_SWIZZLE, a, 3, zxy), op1(AGB_GOP_SWIZZLE, b, 3, yzx)));
            out.n = 3;
            return true;
        }
        if (cat == "rotate2d")
        {
            // MaterialX's rotate2d: (c x + s y, -s x + c y), angle `amount` in degrees.
            if (!in("in", "vector2", "0, 0", a) || !in("amount", "float", "0", b))
                return false;
            Value r  = op2(AGB_GOP_MUL, b, constant({ float(3.14159265358979323846 / 180.0) }, 1));
            Value sn = op1(AGB_GOP_SIN, r), cs = op1(AGB_GOP_COS, r);
            Value x = op1(AGB_GOP_SWIZZLE, a, 1, 0x00), y = op1(AGB_GOP_SWIZZLE, a, 1, 0x55);
            Value rx = op2(AGB_GOP_ADD, op2(AGB_GOP_MUL, cs, x), op2(AGB_GOP_MUL, sn, y));
            Value ry = op2(AGB_GOP_SUB, op2(AGB_GOP_MUL, cs, y), op2(AGB_GOP_MUL, sn, x));
            out = Value{ reg(), 2 };
            emit(AGB_GOP_COMBINE, out.reg, rx.reg, ry.reg, rx.reg, rx.reg, 0);
            return true;
        }
        if (cat == "plus" || cat == "minus" || cat == "difference")
        {
            // MaterialX's compositing nodes (stdlib genglsl): mix x op(fg, bg) + (1 - mix) x bg with
            // op = bg + fg, bg - fg, |bg - fg|.
            Value fg, bg, mx;
            if (!in("fg", type, zero.c_str(), fg) || !in("bg", type, zero.c_str(), bg) || !in("mix", "float", "1", mx))
                return false;
            Value f = cat == "plus" ? op2(AGB_GOP_ADD, bg, fg) : op2(AGB_GOP_SUB, bg, fg);
            if (cat == "difference")
                f = op1(AGB_GOP_ABS, f);
            Value one = valueOf("float", "1", why);
            out       = op2(AGB_GOP_ADD, op2(AGB_GOP_MUL, mx, f), op2(AGB_GOP_MUL, op2(AGB_GOP_SUB, one, mx), bg));
            out.n     = n;
            return true;
        }
        if (cat == "noise2d" || cat == "noise3d" || cat == "fractal3d" || cat == "cellnoise2d" || cat == "cellnoise3d")
        {
            // MaterialX's noise nodes (stdlib genglsl): noise = perlin(p) x amplitude + pivot;
            // fractal3d = amplitude x sum over octaves of diminish^i x perlin(p x lacunarity^i),
            // accumulated in that order; cell noise = the cell's hash in [0, 1].  p: texcoord for
            // the 2D nodes, object-space position for the 3D ones, by default.  Float outputs only
            // (the colour / vector forms hash more channels).
            if (type != "float")
            {
                why = "node <" + cat + "> of type " + type + " is not supported (float only)";
                return false;
            }
            const bool flat = cat == "noise2d" || cat == "cellnoise2d";
            Value pos;
            if (childInput(node, flat ? "texcoord" : "position"))
            {
                if (!in(flat ? "texcoord" : "position", flat ? "vector2" : "vector3", flat ? "0, 0" : "0, 0, 0", pos))
                    return false;
            }
            else
            {
                pos = Value{ reg(), flat ? 2 : 3 };
                emit(AGB_GOP_INPUT, pos.reg, 0, 0, 0, 0, uint16_t(flat ? AGB_GIN_TEXCOORD : AGB_GIN_POSITION_OBJECT));
            }
            auto noise = [&](Value p, int kind) {
                Value r{ reg(), 1 };
                emit(AGB_GOP_NOISE, r.reg, p.reg, 0, 0, 0, uint16_t(kind));
                return r;
            };
            if (cat == "cellnoise2d" || cat == "cellnoise3d")
            {
                out = noise(pos, flat ? 2 : 3);
                return true;
            }
            if (!in("amplitude", "float", "1", a))
                return false;
            if (cat == "fractal3d")
            {
                const XmlElement* oc = childInput(node, "octaves");
                if (oc && !(oc = literalInput(oc, &S)))
                {
                    why = "node <fractal3d> with a connected octaves input is not supported";
                    return false;
                }
                std::vector<float> f = numbers(oc ? oc->attr("value") : "3");
                const int octaves    = f.size() == 1 ? int(f[0]) : -1;
                if (octaves < 0 || octaves > 16)
                {
                    why = "node <fractal3d> octaves must be 0 to 16";
                    return false;
                }
                Value lac, dim;
                if (!in("lacunarity", "float", "2", lac) || !in("diminish", "float", "0.5", dim))
                    return false;
                Value sum = constant({ 0.f }, 1), amp = constant({ 1.f }, 1);
                for (int k = 0; k < octaves; k++)
                {
                    sum = op2(AGB_GOP_ADD, sum, op2(AGB_GOP_MUL, amp, noise(pos, 1)));
                    amp = op2(AGB_GOP_MUL, amp, dim);
                    pos = op2(AGB_GOP_MUL, pos, lac);
                }
                out   = op2(AGB_GOP_MUL, a, sum);
                out.n = 1;
                return true;
            }
            if (!in("pivot", "float", "0", b))
                return false;
            out   = op2(AGB_GOP_ADD, op2(AGB_GOP_MUL, noise(pos, flat ? 0 : 1), a), b);
            out.n = 1;
            return true;
        }
        why = "node <" + cat + "> is not supported";
        return false;
    }
};

// The material field a standard_surface input drives per hit, and its component count.
bool graphField(const std::string& input, int& field, int& n)
{
    static const std::map<std::string, std::pair<int, int>> fields = {
        { "base_color", { AGB_GOUT_BASE_COLOR, 3 } }, { "specular_roughness", { AGB_GOUT_SPECULAR_ROUGHNESS, 1 } },
        { "coat_roughness", { AGB_GOUT_COAT_ROUGHNESS, 1 } }, { "emission_color", { AGB_GOUT_EMISSION_COLOR, 3 } },
        { "opacity", { AGB_GOUT_OPACITY, 3 } }, { "normal", { AGB_GOUT_NORMAL, 3 } }
    };
    auto it = fields.find(input);
    if (it == fields.end())
        return false;
    field = it->second.first;
    n     = it->second.second;
    return true;
}

// An adsk compound surface shader as the standard_surface it stands for: `out` receives copies of
// the compound's inputs renamed to the Standard Surface inputs they drive (the reference's map of
// compound interface inputs to material fields, MaterialX/MaterialGenerator.cpp:90-114), and
// `constants` the values the compound fixes inside: metalness 1 for adsk:metal
// (BSDFCodeGenerator.cpp:1525), transmission 1 for adsk:transparent (BSDFCodeGenerator.cpp:540),
// thin_walled for adsk:glazing (BSDFCodeGenerator.cpp:1525-1526; a glazing is a thin
// transmissive layer, so transmission 1 too: the reference counts a glazing_transmission_color as
// non-opaque, MaterialGenerator.cpp:365-368); and for adsk:opaque, emission 1 when
// opaque_emission is set with a positive opaque_luminance and subsurface 1 with
// opaque_translucency (MaterialGenerator.cpp:315-333).
bool adskCompound(const XmlElement& shader, XmlElement& out, Properties& constants)
{
    static const std::map<std::string, std::string> inputMap = {
        { "layered_diffuse", "base_color" }, { "layered_roughness", "specular_roughness" },
        { "layered_fraction", "coat" }, { "layered_anisotropy", "specular_anisotropy" },
        { "layered_rotation", "specular_rotation" }, { "layered_normal", "normal" },
        { "layered_bottom_f0", "specular_color" }, { "opaque_albedo", "base_color" }, { "metal_f0", "base_color" },
        { "surface_roughness", "specular_roughness" }, { "surface_anisotropy", "specular_anisotropy" },
        { "surface_rotation", "specular_rotation" }, { "surface_albedo", "coat_color" },
        { "surface_normal", "normal" }, { "surface_cutout", "opacity" }, { "transparent_ior", "specular_IOR" },
        { "transparent_color", "transmission_color" }, { "glazing_transmission_color", "transmission_color" },
        { "glazing_transmission_roughness", "specular_roughness" }, { "glazing_f0", "specular_color" },
        { "opaque_luminance_modifier", "emission_color" }, { "opaque_mfp_modifier", "subsurface_color" },
    };
    const std::string kind = shader.name;
    if (kind != "adsk:opaque" && kind != "adsk:metal" && kind != "adsk:transparent" && kind != "adsk:glazing" &&
        kind != "adsk:layered")
        return false;
    out.name  = "standard_surface";
    out.attrs = shader.attrs;
    auto value = [&](const char* name) -> std::string {
        for (auto& c : shader.children)
            if (c->name == "input" && c->attr("name") == name)
                return c->attr("value");
        return std::string();
    };
    for (auto& c : shader.children)
    {
        if (c->name != "input")
            continue;
        auto it = inputMap.find(c->attr("name"));
        if (it == inputMap.end())
            continue;
        auto copy           = std::make_unique<XmlElement>();
        copy->name          = c->name;
        copy->attrs         = c->attrs;
        copy->attrs["name"] = it->second;
        out.children.push_back(std::move(copy));
    }
    if (kind == "adsk:metal")
        constants["metalness"] = 1.f;
    else if (kind == "adsk:transparent")
        constants["transmission"] = 1.f;
    else if (kind == "adsk:glazing")
    {
        constants["thin_walled"]  = true;
        constants["transmission"] = 1.f;
    }
    else if (kind == "adsk:opaque")
    {
        const std::string e = value("opaque_emission"), t = value("opaque_translucency");
        std::vector<float> lum = numbers(value("opaque_luminance"));
        if ((e == "true" || e == "1") && lum.size() == 1 && lum[0] > 0.f)
            constants["emission"] = 1.f;
        if (t == "true" || t == "1")
            constants["subsurface"] = 1.f;
    }
    return true;
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
    // Autodesk's compound surface shaders (Prism materials) drive the Standard Surface fields
    // their interface inputs map to; inputs outside the map are not used.
    XmlElement compound;
    Properties compoundConstants;
    if (shader->name != "standard_surface")
    {
        if (!adskCompound(*shader, compound, compoundConstants))
        {
            warnings += "MaterialX document: surface shader <" + shader->name +
                "> is not supported (only standard_surface and the adsk:opaque, adsk:metal, adsk:transparent, "
                "adsk:glazing and adsk:layered compounds)\n";
            return false;
        }
        shader = &compound;
    }
    const std::string docSpace = root.has("colorspace") ? root.attr("colorspace") : "lin_rec709";
    GraphCompiler graphs(root, baseDirectory, docSpace, warnings, images);
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
            int field = 0, comps = 0;
            if (graphField(n, field, comps))
                graphs.compileOutput(*in, field, comps);
            else
                warnings += "MaterialX input '" + n + "' is connected to a node graph, which drives only base_color, " +
                    "specular_roughness, coat_roughness, emission_color, opacity and normal per hit; its default is used\n";
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
    for (auto& kv : compoundConstants)
        properties[kv.first] = kv.second;
    Strings program;
    if (!graphs.empty())
    {
        if (graphs.program(program))
            properties["materialx_graph"] = program;
        else
            warnings += "MaterialX node graphs need more than " + std::to_string(AGB_GRAPH_REGS) +
                " values at once; their inputs keep their defaults\n";
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
