#pragma once
#include "imageio.h"
namespace OIIO {
struct ustring {
    std::string s;
    ustring() {}
    ustring(const std::string &x) : s(x) {}
    std::string string() const { return s; }
};
inline std::ostream &operator<<(std::ostream &o, const ustring &u) { return o << u.s; }
struct TextureOpt {
    enum class Wrap { WrapPeriodic };
    Wrap swrap, twrap;
};
class TextureSystem {
  public:
    static TextureSystem *create() { return new TextureSystem(); }
    static void destroy(TextureSystem *t) { delete t; }
    bool attribute(const std::string &, int) { return true; }
    bool texture(const ustring &, TextureOpt &, float, float, float, float, float, float,
                 int, float *) { return false; }
};
}  // namespace OIIO
