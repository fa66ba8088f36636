// The reference's frame.cpp (the Qt OpenGL widget and QImage writer) does not build here; this
// file gives the plain if_frame base a headless definition so the reference's compositors can
// commit into a memory frame: one surface per buffer, pixels indexed i + j * w of the back one.
#include "frame.h"

e8::if_frame::surface::surface() {}

e8::if_frame::surface::~surface() {}

void e8::if_frame::surface::resize(unsigned nw, unsigned nh) {
    w = nw;
    h = nh;
    pixels = std::make_unique<pixel[]>(static_cast<size_t>(nw) * nh);
}

e8::if_frame::if_frame() {}

e8::if_frame::~if_frame() {}

e8::if_frame::surface &e8::if_frame::back() { return m_surface[m_spin]; }

e8::pixel &e8::if_frame::operator()(unsigned i, unsigned j) { return back().pixels[i + j * back().w]; }
