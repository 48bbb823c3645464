// PFM-only image input/output behind the OpenImageIO names the reference uses.
// Test infrastructure for the oracle build of the reference (never shipped).
// Reference call sites: src/image.cpp:5-58 (Image3 from file, WriteImage).
#include <OpenImageIO/imageio.h>
#include <cstring>
#include <vector>

namespace OIIO {

std::string geterror() { return "oiio shim: PFM only"; }

std::unique_ptr<ImageInput> ImageInput::open(const std::string &filename) {
    FILE *f = fopen(filename.c_str(), "rb");
    if (!f) return nullptr;
    char magic[3] = {0, 0, 0};
    int w, h;
    double scale;
    if (fscanf(f, "%2s %d %d %lf", magic, &w, &h, &scale) != 4) { fclose(f); return nullptr; }
    fgetc(f);  // single whitespace after header
    std::unique_ptr<ImageInput> in(new ImageInput());
    in->m_file = f;
    in->m_spec = ImageSpec(w, h, std::strcmp(magic, "PF") == 0 ? 3 : 1, TypeDesc::FLOAT);
    in->m_littleEndian = scale < 0;
    return in;
}

bool ImageInput::read_image(TypeDesc format, void *data) {
    const size_t n = size_t(m_spec.width) * m_spec.height * m_spec.nchannels;
    std::vector<float> buf(n);
    if (fread(buf.data(), sizeof(float), n, m_file) != n) return false;
    // PFM rows are stored bottom to top.
    const size_t row = size_t(m_spec.width) * m_spec.nchannels;
    for (int y = 0; y < m_spec.height; y++) {
        const float *src = &buf[size_t(m_spec.height - 1 - y) * row];
        for (size_t i = 0; i < row; i++) {
            if (format == TypeDesc::DOUBLE) ((double *)data)[y * row + i] = src[i];
            else ((float *)data)[y * row + i] = src[i];
        }
    }
    return true;
}

void ImageInput::close() {
    if (m_file) fclose(m_file);
    m_file = nullptr;
}

ImageInput::~ImageInput() { close(); }

std::unique_ptr<ImageOutput> ImageOutput::create(const std::string &filename) {
    return std::unique_ptr<ImageOutput>(new ImageOutput());
}

bool ImageOutput::open(const std::string &filename, const ImageSpec &spec) {
    m_name = filename;
    m_spec = spec;
    return true;
}

bool ImageOutput::write_image(TypeDesc format, const void *data) {
    // Whatever extension was asked for, the pixels are written as PFM next to it.
    std::string name = m_name;
    size_t dot = name.rfind('.');
    if (dot != std::string::npos) name = name.substr(0, dot);
    name += ".pfm";
    FILE *f = fopen(name.c_str(), "wb");
    if (!f) return false;
    fprintf(f, "PF\n%d %d\n-1.0\n", m_spec.width, m_spec.height);
    const size_t row = size_t(m_spec.width) * 3;
    std::vector<float> buf(row);
    for (int y = m_spec.height - 1; y >= 0; y--) {
        for (size_t i = 0; i < row; i++) {
            buf[i] = format == TypeDesc::DOUBLE ? float(((const double *)data)[y * row + i])
                                                : ((const float *)data)[y * row + i];
        }
        fwrite(buf.data(), sizeof(float), row, f);
    }
    fclose(f);
    return true;
}

void ImageOutput::close() {}

}  // namespace OIIO
