// ps_params.cpp -- camera parameter files: the PTGui .pts reader of
// loadPhotoParams (source/Warp/PhotoParam.cpp:756-771, loadPhotoParamFromPTS
// :681-754 with its line parsers :513-678), restated on the host.  The XML
// reader of the reference needs the ticpp library and is not built.
#include <cstring>
#include <fstream>
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

}  // namespace

std::vector<ps_photo_param> loadPhotoParams(const std::string& path)
{
    const size_t dot = path.find_last_of('.');
    if (dot == std::string::npos) fail(PS_EINVAL, "%s: the file has no extension", path.c_str());
    if (path.substr(dot + 1) != "pts")
        fail(PS_EINVAL, "%s: only PTGui .pts camera files are read (the XML reader needs ticpp)", path.c_str());
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
