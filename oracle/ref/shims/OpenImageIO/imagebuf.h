#pragma once
#include "texture.h"
#include <stdexcept>
namespace OIIO {
class ImageBuf {
  public:
    ImageBuf(const ustring &) { throw std::runtime_error("bitmap textures unsupported in oracle build"); }
    ImageSpec nativespec() const { return ImageSpec(); }
    int nchannels() const { return 0; }
};
}  // namespace OIIO
