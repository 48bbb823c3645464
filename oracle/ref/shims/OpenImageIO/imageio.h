#pragma once
#include "oiioversion.h"
#include <memory>
#include <string>
#include <cstdio>
namespace OIIO {
struct TypeDesc {
    enum BASETYPE { UNKNOWN, UINT8, HALF, FLOAT, DOUBLE };
    BASETYPE basetype;
    TypeDesc(BASETYPE b = UNKNOWN) : basetype(b) {}
    bool operator==(const TypeDesc &o) const { return basetype == o.basetype; }
    bool operator==(BASETYPE b) const { return basetype == b; }
};
struct ImageSpec {
    int width = 0, height = 0, nchannels = 0;
    TypeDesc format;
    ImageSpec() {}
    ImageSpec(int w, int h, int c, TypeDesc f) : width(w), height(h), nchannels(c), format(f) {}
};
class ImageInput {
  public:
    static std::unique_ptr<ImageInput> open(const std::string &filename);
    const ImageSpec &spec() const { return m_spec; }
    bool read_image(TypeDesc format, void *data);
    void close();
    ~ImageInput();
  private:
    ImageSpec m_spec;
    FILE *m_file = nullptr;
    bool m_littleEndian = true;
};
class ImageOutput {
  public:
    static std::unique_ptr<ImageOutput> create(const std::string &filename);
    bool open(const std::string &filename, const ImageSpec &spec);
    bool write_image(TypeDesc format, const void *data);
    void close();
  private:
    std::string m_name;
    ImageSpec m_spec;
};
std::string geterror();
}  // namespace OIIO
