// ps_params.cpp -- camera parameter files, as loadPhotoParams reads them
// (source/Warp/PhotoParam.cpp:756-771): the PTGui .pts reader
// (loadPhotoParamFromPTS :681-754 with its line parsers :513-678) and the XML
// reader (loadPhotoParamFromXML :17-506), restated on the host.  The
// reference reads XML through the ticpp library; here a small reader of our
// own parses the element tree (elements, text, attributes, comments,
// declarations), and the two layouts the reference accepts are read from it.
#include <cctype>
#include <cstring>
#include <fstream>
#include <initializer_list>
#include <sstream>
#include <string>
#include <vector>

#include "ps_internal.h"

namespace ps {
namespace {

bool infoLine(const std::string& line) { return !line.empty() && line[0] != '#'; }

// The text from `begin` to the line's first space, or to the end of the line
// when that space comes before `begin` (the reference's getValueString).
std::string valueText(const std::string& line, size_t begin)
{
    const size_t space = line.find(' ');
    if (space == std::string::npos || space < begin) return line.substr(begin);
    return line.substr(begin, space - begin);
}

// The number a stream extraction reads from the start of s; 0 when none.
double leadingNumber(const std::string& s)
{
    std::istringstream in(s);
    double v = 0;
    if (!(in >> v)) v = 0;
    return v;
}

double valueAfter(const std::string& line, size_t key) { return leadingNumber(valueText(line, key + 1)); }

// Comma-separated numbers after `key` (the reference's getValues).
std::vector<double> valuesAfter(const std::string& line, size_t key)
{
    const std::string text = valueText(line, key + 1);
    std::vector<double> out;
    size_t from = 0;
    while (true) {
        const size_t comma = text.find(',', from);
        out.push_back(leadingNumber(text.substr(from, comma == std::string::npos ? std::string::npos : comma - from)));
        if (comma == std::string::npos) break;
        from = comma + 1;
    }
    return out;
}

// The global "o" line: hfov v, distortion a b c, shift d e, shear g t
// (tryParseGlobalPhotoParam).  Every key is the first occurrence of its
// letter anywhere in the line.
bool parseGlobal(const std::string& line, ps_photo_param& p)
{
    if (line.empty() || line[0] != 'o') return false;
    const char keys[] = "vabcdegt";
    size_t pos[8];
    for (int k = 0; k < 8; k++)
        if ((pos[k] = line.find(keys[k])) == std::string::npos) return false;
    std::memset(&p, 0, sizeof p);
    p.hfov = valueAfter(line, pos[0]);
    p.alpha = valueAfter(line, pos[1]);
    p.beta = valueAfter(line, pos[2]);
    p.gamma = valueAfter(line, pos[3]);
    p.shift_x = valueAfter(line, pos[4]);
    p.shift_y = valueAfter(line, pos[5]);
    p.shear_x = valueAfter(line, pos[6]);
    p.shear_y = valueAfter(line, pos[7]);
    return true;
}

// A camera "o" line: PanoTools projection f, yaw y, pitch p, roll r and the
// optional crop C left,right,top,bottom (tryParseIndividualPhotoParam).
bool parseCamera(const std::string& line, ps_photo_param& p)
{
    if (line.empty() || line[0] != 'o') return false;
    const size_t f = line.find('f'), y = line.find('y'), pp = line.find('p'), r = line.find('r'), c = line.find('C');
    if (f == std::string::npos || y == std::string::npos || pp == std::string::npos || r == std::string::npos)
        return false;
    std::memset(&p, 0, sizeof p);
    // PanoTools 0 rectilinear, 2 circular fisheye, 3 full-frame fisheye ->
    // image types 0, 3, 1; anything else stays rectilinear
    const int pt = (int)(valueAfter(line, f) + 0.5);
    if (pt == 2) p.image_type = 3;
    else if (pt == 3) p.image_type = 1;
    p.yaw = valueAfter(line, y);
    p.pitch = valueAfter(line, pp);
    p.roll = valueAfter(line, r);
    if (c != std::string::npos) {
        const std::vector<double> v = valuesAfter(line, c);
        if (v.size() != 4) return false;
        p.crop_x = (int)v[0];
        p.crop_y = (int)v[2];
        p.crop_width = (int)(v[1] - v[0]);
        p.crop_height = (int)(v[3] - v[2]);
    }
    return true;
}

// ---- XML ------------------------------------------------------------------
struct XmlNode {
    std::string name;
    std::string text;  // the element's first run of character data
    std::vector<XmlNode> children;
};

// A minimal well-formedness-checking reader of the element tree.
class XmlReader {
public:
    explicit XmlReader(const std::string& s) : s_(s) {}
    bool parse(std::vector<XmlNode>& top)
    {
        while (true) {
            skipMisc();
            if (pos_ >= s_.size()) return true;
            if (s_[pos_] != '<') return false;  // text outside the root elements
            XmlNode n;
            if (!element(n)) return false;
            top.push_back(std::move(n));
        }
    }

private:
    // whitespace, comments, declarations and processing instructions
    void skipMisc()
    {
        while (pos_ < s_.size()) {
            if (std::isspace((unsigned char)s_[pos_])) {
                pos_++;
            } else if (s_.compare(pos_, 4, "<!--") == 0) {
                const size_t e = s_.find("-->", pos_ + 4);
                pos_ = e == std::string::npos ? s_.size() : e + 3;
            } else if (s_.compare(pos_, 2, "<?") == 0) {
                const size_t e = s_.find("?>", pos_ + 2);
                pos_ = e == std::string::npos ? s_.size() : e + 2;
            } else if (s_.compare(pos_, 2, "<!") == 0 && s_.compare(pos_, 9, "<![CDATA[") != 0) {
                const size_t e = s_.find('>', pos_ + 2);
                pos_ = e == std::string::npos ? s_.size() : e + 1;
            } else {
                return;
            }
        }
    }
    bool nameAt(std::string& out)
    {
        const size_t b = pos_;
        while (pos_ < s_.size() && !std::isspace((unsigned char)s_[pos_]) && s_[pos_] != '>' && s_[pos_] != '/')
            pos_++;
        out = s_.substr(b, pos_ - b);
        return !out.empty();
    }
    bool element(XmlNode& n)
    {
        pos_++;  // '<'
        if (!nameAt(n.name)) return false;
        // attributes (ignored), up to '>' or '/>'
        char quote = 0;
        while (pos_ < s_.size()) {
            const char c = s_[pos_];
            if (quote) {
                if (c == quote) quote = 0;
            } else if (c == '"' || c == '\'') {
                quote = c;
            } else if (c == '>') {
                break;
            } else if (c == '/' && pos_ + 1 < s_.size() && s_[pos_ + 1] == '>') {
                pos_ += 2;
                return true;  // empty element
            }
            pos_++;
        }
        if (pos_ >= s_.size()) return false;
        pos_++;  // '>'
        bool haveText = false;
        while (pos_ < s_.size()) {
            if (s_[pos_] != '<') {  // character data
                const size_t e = s_.find('<', pos_);
                const std::string t = s_.substr(pos_, (e == std::string::npos ? s_.size() : e) - pos_);
                if (!haveText && t.find_first_not_of(" \t\r\n") != std::string::npos) {
                    n.text = t;
                    haveText = true;
                }
                pos_ = e == std::string::npos ? s_.size() : e;
            } else if (s_.compare(pos_, 2, "</") == 0) {
                pos_ += 2;
                std::string close;
                if (!nameAt(close) || close != n.name) return false;
                while (pos_ < s_.size() && std::isspace((unsigned char)s_[pos_])) pos_++;
                if (pos_ >= s_.size() || s_[pos_] != '>') return false;
                pos_++;
                return true;
            } else if (s_.compare(pos_, 9, "<![CDATA[") == 0) {
                const size_t e = s_.find("]]>", pos_ + 9);
                if (e == std::string::npos) return false;
                if (!haveText) {
                    n.text = s_.substr(pos_ + 9, e - pos_ - 9);
                    haveText = true;
                }
                pos_ = e + 3;
            } else if (s_.compare(pos_, 4, "<!--") == 0 || s_.compare(pos_, 2, "<?") == 0) {
                skipMisc();
            } else {
                XmlNode c;
                if (!element(c)) return false;
                n.children.push_back(std::move(c));
            }
        }
        return false;  // unclosed
    }

    const std::string& s_;
    size_t pos_ = 0;
};

const XmlNode* firstChild(const XmlNode& n, const char* name)
{
    for (const XmlNode& c : n.children)
        if (c.name == name) return &c;
    return nullptr;
}

// The elements named `name` among n's children, in order (ticpp's sibling
// iteration from the first of them).
std::vector<const XmlNode*> childrenNamed(const XmlNode& n, const char* name)
{
    std::vector<const XmlNode*> out;
    for (const XmlNode& c : n.children)
        if (c.name == name) out.push_back(&c);
    return out;
}

// GetText(&double): the number a stream extraction reads from the element's
// text; a missing element or text without a leading number fails the layout.
bool number(const XmlNode& parent, const char* name, double& v)
{
    const XmlNode* e = firstChild(parent, name);
    if (!e) return false;
    std::istringstream in(e->text);
    return static_cast<bool>(in >> v);
}

struct Field {
    const char* name;
    double* value;
};

bool numbers(const XmlNode& parent, std::initializer_list<Field> fields)
{
    for (const Field& f : fields)
        if (!number(parent, f.name, *f.value)) return false;
    return true;
}

// The camera elements of a Root: its POSITION children, else its VIDEO ones.
std::vector<const XmlNode*> cameraNodes(const XmlNode& root)
{
    std::vector<const XmlNode*> v = childrenNamed(root, "POSITION");
    return v.empty() ? childrenNamed(root, "VIDEO") : v;
}

// loadPhotoParamFromXML2 (:261-496): one Root whose camera elements carry
// every field.
bool xmlLayoutPerCamera(const std::vector<XmlNode>& top, std::vector<ps_photo_param>& params)
{
    params.clear();
    const XmlNode* root = nullptr;
    for (const XmlNode& n : top)
        if (n.name == "Root") {
            root = &n;
            break;
        }
    if (!root) return false;
    const std::vector<const XmlNode*> cams = cameraNodes(*root);
    if (cams.empty()) return false;
    for (const XmlNode* c : cams) {
        double type, cropMode, hfov, vfov, a, b, g, sx, sy, hx, hy, l, r, t, bo, cx, cy, cr, yaw, pitch, roll;
        if (!numbers(*c, {{"IMAGETYPE", &type}, {"CROPMODE", &cropMode}, {"HFOV", &hfov}, {"VFOV", &vfov},
                          {"Alpha", &a}, {"Beta", &b}, {"Gamma", &g}, {"ShiftX", &sx}, {"ShiftY", &sy},
                          {"ShearX", &hx}, {"ShearY", &hy}, {"CROPLEFT", &l}, {"CROPRIGHT", &r}, {"CROPTOP", &t},
                          {"CROPBOTTOM", &bo}, {"CircleX", &cx}, {"CircleY", &cy}, {"CircleR", &cr},
                          {"YAW", &yaw}, {"PITCH", &pitch}, {"ROLL", &roll}})) {
            params.clear();
            return false;
        }
        ps_photo_param p;
        std::memset(&p, 0, sizeof p);
        p.image_type = (int)type;
        p.crop_mode = (int)cropMode;
        p.hfov = hfov;
        p.vfov = vfov;
        p.alpha = a;
        p.beta = b;
        p.gamma = g;
        p.shift_x = sx;
        p.shift_y = sy;
        p.shear_x = hx;
        p.shear_y = hy;
        p.crop_x = (int)l;
        p.crop_width = (int)(r - p.crop_x);  // the int field, as the reference subtracts it
        p.crop_y = (int)t;
        p.crop_height = (int)(bo - p.crop_y);
        p.circle_x = (int)cx;
        p.circle_y = (int)cy;
        p.circle_r = (int)cr;
        p.yaw = yaw;
        p.pitch = pitch;
        p.roll = roll;
        params.push_back(p);
    }
    return true;
}

// loadPhotoParamFromXML1 (:17-259): Root elements each holding a GlobalInfo
// (lens, optional crop) and camera elements with the pose (and the crop when
// GlobalInfo has none).
bool xmlLayoutGlobalInfo(const std::vector<XmlNode>& top, std::vector<ps_photo_param>& params)
{
    params.clear();
    std::vector<const XmlNode*> roots;
    for (const XmlNode& n : top)
        if (n.name == "Root") roots.push_back(&n);
    if (roots.empty()) return false;
    for (const XmlNode* root : roots) {
        ps_photo_param p;
        std::memset(&p, 0, sizeof p);
        const XmlNode* gi = firstChild(*root, "GlobalInfo");
        if (!gi) {
            params.clear();
            return false;
        }
        double type, cropMode, l, r, t, bo;
        if (!numbers(*gi, {{"IMAGETYPE", &type}, {"CROPMODE", &cropMode}, {"HFOV", &p.hfov}, {"VFOV", &p.vfov}})) {
            params.clear();
            return false;
        }
        p.image_type = (int)type;
        p.crop_mode = (int)cropMode;
        const bool cropInRoot = firstChild(*gi, "CROPLEFT") != nullptr;
        if (cropInRoot) {
            if (!numbers(*gi, {{"CROPLEFT", &l}, {"CROPRIGHT", &r}, {"CROPTOP", &t}, {"CROPBOTTOM", &bo}})) {
                params.clear();
                return false;
            }
            p.crop_x = (int)l;
            p.crop_width = (int)(r - p.crop_x);
            p.crop_y = (int)t;
            p.crop_height = (int)(bo - p.crop_y);
        }
        if (!numbers(*gi, {{"Alpha", &p.alpha}, {"Beta", &p.beta}, {"Gamma", &p.gamma}, {"ShiftX", &p.shift_x},
                           {"ShiftY", &p.shift_y}, {"ShearX", &p.shear_x}, {"ShearY", &p.shear_y}})) {
            params.clear();
            return false;
        }
        const std::vector<const XmlNode*> cams = cameraNodes(*root);
        if (cams.empty()) {
            params.clear();
            return false;
        }
        for (const XmlNode* c : cams) {
            if (!cropInRoot) {
                if (!numbers(*c, {{"CROPLEFT", &l}, {"CROPRIGHT", &r}, {"CROPTOP", &t}, {"CROPBOTTOM", &bo}})) {
                    params.clear();
                    return false;
                }
                p.crop_x = (int)l;
                p.crop_width = (int)(r - p.crop_x);
                p.crop_y = (int)t;
                p.crop_height = (int)(bo - p.crop_y);
            }
            if (!numbers(*c, {{"YAW", &p.yaw}, {"PITCH", &p.pitch}, {"ROLL", &p.roll}})) {
                params.clear();
                return false;
            }
            params.push_back(p);
        }
    }
    return true;
}

// loadPhotoParamFromXML (:498-503): the per-camera layout first, then the
// GlobalInfo one; an unreadable file gives no cameras.
std::vector<ps_photo_param> loadXml(const std::string& path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in.is_open()) fail(PS_EINVAL, "%s: cannot open", path.c_str());
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
    std::vector<XmlNode> top;
    XmlReader reader(text);
    std::vector<ps_photo_param> params;
    if (!reader.parse(top)) return params;
    if (xmlLayoutPerCamera(top, params)) return params;
    xmlLayoutGlobalInfo(top, params);
    return params;
}

}  // namespace

std::vector<ps_photo_param> loadPhotoParams(const std::string& path)
{
    const size_t dot = path.find_last_of('.');
    if (dot == std::string::npos) fail(PS_EINVAL, "%s: the file has no extension", path.c_str());
    if (path.substr(dot + 1) != "pts") return loadXml(path);  // any other extension is XML, as in the reference
    std::ifstream in(path);
    if (!in.is_open()) fail(PS_EINVAL, "%s: cannot open", path.c_str());
    std::vector<ps_photo_param> params;
    std::string line;
    bool valid = false;
    while (std::getline(in, line))
        if (line.find("ptGui project file") != std::string::npos) {
            valid = true;
            break;
        }
    if (!valid) return params;
    ps_photo_param global;
    bool globalSet = false;
    while (std::getline(in, line)) {
        if (!infoLine(line)) continue;
        if (!globalSet && (globalSet = parseGlobal(line, global))) continue;  // the global line is not a camera
        ps_photo_param cam;
        if (parseCamera(line, cam)) params.push_back(cam);
    }
    if (!globalSet) return {};
    for (ps_photo_param& p : params) {
        p.hfov = global.hfov;
        p.alpha = global.alpha;
        p.beta = global.beta;
        p.gamma = global.gamma;
        p.shift_x = global.shift_x;
        p.shift_y = global.shift_y;
        p.shear_x = global.shear_x;
        p.shear_y = global.shear_y;
    }
    return params;
}

}  // namespace ps
