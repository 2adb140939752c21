// Shading and blending of one fragment: the brushes of
// src/render/sw/sw_span_brush.cc (solid :140-152, linear/radial gradients
// :164-383, pixmap nearest :555-579 with src/graphic/bitmap_sampler.cc) and
// SWRenderTarget::BlendPixel with FastBlend (sw_render_target.cc:12-141),
// premultiplied ARGB arithmetic of src/graphic/color_priv.hpp:20-72.
#pragma once
#include "geom.cuh"

namespace skc {

// Per-pass brush, prepared on the host the way SWCanvas::GenerateBrush
// (sw_canvas.cc:727-795) prepares the reference's SWSpanBrush.
struct Brush {
  uint32_t kind;          // 0 solid, 1 linear, 2 radial, 3 image (blur mask), 4 sweep, 5 conical,
                          // 6 image shader (tile: ImageMode)
  uint32_t blend;         // BlendMode
  uint32_t solid;         // premultiplied ARGB (kind 0)
  uint32_t global_alpha;  // SWSpanBrush::global_alpha_ (255 except image)
  float m[6];             // sx, kx, tx, ky, sy, ty of the device->unit matrix
  uint32_t tile, stop_count, has_offsets, stop0;  // gradient stops
  uint32_t img_w, img_h;  // image brush source
  uint64_t img_off;       // byte offset of the source pixels (RGBA8 rows)
  float bias, scale;      // sweep: GradientInfo::radius (bias, scale of the angle)
  uint32_t conical;       // conical: index of its ConicalParams
  uint32_t cf_type;       // colour filter: 0 none, 1 blend, 2 matrix, 3 linear->sRGB,
                          // 4 sRGB->linear (compose is the identity on this path)
  uint32_t cf_mode;       // blend filter: BlendMode
  uint32_t cf_pm;         // blend filter: its colour, premultiplied
  uint32_t cf_index;      // matrix filter: first of its 20 int16 terms in DevBatch::cf_matrices
  uint32_t pad;
};

// ConicalGradientColorBrush after OnPreBrush (sw_span_brush.cc:394-437),
// prepared on the host; MapPoint form of the matrices (sx, kx, tx, ky, sy, ty).
struct ConicalParams {
  float d2l[6];           // device_to_local, applied first
  float t[6];             // then c0 -> c1 (strip) or cf -> c1 (general) to unit
  float c0x, c0y;         // radial: start centre
  float scale, scale_sign, bias;  // radial
  float r2;               // strip: (r0 / |c1 - c0|)^2
  float f, r1, r1_square; // general
  uint32_t mode;          // 0 transparent (a negative radius), 1 radial, 2 radial with equal
                          // radii (transparent), 3 strip, 4 general
  uint32_t swap01;        // general: the ends were swapped (t -> 1 - t)
  uint32_t pad;
};

SKC_HD uint32_t GetA(uint32_t c) { return (c >> 24) & 0xFF; }
SKC_HD uint32_t ARGB(uint32_t a, uint32_t r, uint32_t g, uint32_t b) {
  return (a << 24) | (r << 16) | (g << 8) | b;
}
// RGBA8 bytes in memory (little-endian u32 R | G<<8 | B<<16 | A<<24) <-> ARGB
SKC_HD uint32_t RGBAtoARGB(uint32_t m) {
  return (m & 0xFF00FF00u) | ((m & 0xFFu) << 16) | ((m >> 16) & 0xFFu);
}
SKC_HD uint32_t ARGBtoRGBA(uint32_t c) { return RGBAtoARGB(c); }  // same swap

SKC_HD uint8_t ChannelToByte(float v) {  // Color4fToColor (color.cc:53-59)
  float s = v * 255;
  s = min_(max_(s, 0.f), 255.f);
  return (uint8_t)s;
}
SKC_HD uint32_t Color4fToColor(float r, float g, float b, float a) {
  return ARGB(ChannelToByte(a), ChannelToByte(r), ChannelToByte(g), ChannelToByte(b));
}
SKC_HD uint32_t MulDiv255Round(uint32_t a, uint32_t b) {  // color_priv.hpp:31-47
  uint32_t prod = a * b + 128;
  return (prod + (prod >> 8)) >> 8;
}
SKC_HD uint32_t ColorToPMColor(uint32_t c) {  // color_priv.cc:105-108
  uint32_t a = GetA(c), r = (c >> 16) & 0xFF, g = (c >> 8) & 0xFF, b = c & 0xFF;
  if (a != 255) {
    r = MulDiv255Round(r, a);
    g = MulDiv255Round(g, a);
    b = MulDiv255Round(b, a);
  }
  return (a << 24) | (r << 16) | (g << 8) | b;
}
SKC_HD uint32_t AlphaMulQ(uint32_t c, uint32_t scale) {  // color_priv.hpp:62-68
  const uint32_t mask = 0xFF00FF;
  uint32_t rb = ((c & mask) * scale) >> 8;
  uint32_t ag = ((c >> 8) & mask) * scale;
  return (rb & mask) | (ag & ~mask);
}
SKC_HD uint32_t PMSrcOver(uint32_t src, uint32_t dst) {  // color_priv.hpp:70-72
  return src + AlphaMulQ(dst, 256 - GetA(src));
}

SKC_HD uint32_t GetR(uint32_t c) { return (c >> 16) & 0xFF; }
SKC_HD uint32_t GetG(uint32_t c) { return (c >> 8) & 0xFF; }
SKC_HD uint32_t GetB(uint32_t c) { return c & 0xFF; }
SKC_HD uint32_t PMColorMul(uint32_t s, uint32_t d) {  // color_priv.hpp:74-79
  return (MulDiv255Round(GetA(s), GetA(d)) << 24) | (MulDiv255Round(GetR(s), GetR(d)) << 16) |
         (MulDiv255Round(GetG(s), GetG(d)) << 8) | MulDiv255Round(GetB(s), GetB(d));
}

// SoftLight of one channel (blend_mode.cc:91-108): s = (colour, alpha) of
// the source, d of the destination, as fractions of 255.
SKC_HD float SoftLightChannel(float sc, float sa, float dc, float da) {
  if (2.f * sc <= sa) {
    return dc * dc * (sa - 2 * sc) / da + (1 - da) * sc + dc * (-sa + 2 * sc + 1);
  }
  if (4.f * dc <= da) {
    const float d2 = dc * dc, d3 = d2 * dc, a2 = da * da, a3 = a2 * da;
    return (a2 * (sc - dc * (3 * sa - 6 * sc - 1)) + 12 * da * d2 * (sa - 2 * sc) -
            16 * d3 * (sa - 2 * sc) - a3 * sc) /
           a2;
  }
  return dc * (sa - 2 * sc + 1) + sc - sqrt_(da * dc) * (sa - 2 * sc) - da * sc;
}

// PorterDuffBlend (blend_mode.cc:123-191): the coefficient modes up to
// kScreen and kSoftLight; any other mode blends as kSrcOver (kDefault).
SKC_HD uint32_t PorterDuff(uint32_t src, uint32_t dst, uint32_t mode) {
  if (mode > 14 && mode != 21) mode = 3;
  const uint32_t sa = GetA(src), da = GetA(dst);
  switch (mode) {
    case 0: return 0;
    case 1: return src;
    case 2: return dst;
    case 3: return sa == 0 ? dst : PMSrcOver(src, dst);
    case 4: return da == 255 ? dst : PMSrcOver(dst, src);                    // kDstOver
    case 5: return da == 255 ? src : AlphaMulQ(src, da + 1);                // kSrcIn
    case 6: return sa == 255 ? dst : AlphaMulQ(dst, sa + 1);                // kDstIn
    case 7: return da == 0 ? src : AlphaMulQ(src, 256 - da);                // kSrcOut
    case 8: return sa == 0 ? dst : AlphaMulQ(dst, 256 - sa);                // kDstOut
    case 9: return AlphaMulQ(src, da + 1) + AlphaMulQ(dst, 256 - sa);       // kSrcATop
    case 10: return AlphaMulQ(dst, sa + 1) + AlphaMulQ(src, 256 - da);      // kDstATop
    case 11: return AlphaMulQ(src, 256 - da) + AlphaMulQ(dst, 256 - sa);    // kXor
    case 12:                                                                 // kPlus
      return ARGB(min_(sa + da, 255u), min_(GetR(src) + GetR(dst), 255u),
                  min_(GetG(src) + GetG(dst), 255u), min_(GetB(src) + GetB(dst), 255u));
    case 13: return PMColorMul(src, dst);                                    // kModulate
    case 14: return src + dst - PMColorMul(src, dst);                        // kScreen
    default: {                                                               // kSoftLight
      if (da == 0) return src;
      // Color4fFromColor (color.cc:44-51)
      const float s_r = GetR(src) / 255.f, s_g = GetG(src) / 255.f, s_b = GetB(src) / 255.f;
      const float s_a = sa / 255.f;
      const float d_r = GetR(dst) / 255.f, d_g = GetG(dst) / 255.f, d_b = GetB(dst) / 255.f;
      const float d_a = da / 255.f;
      const float r = SoftLightChannel(s_r, s_a, d_r, d_a);
      const float g = SoftLightChannel(s_g, s_a, d_g, d_a);
      const float b = SoftLightChannel(s_b, s_a, d_b, d_a);
      const float a = s_a + (1 - s_a) * d_a;
      return Color4fToColor(r, g, b, a);
    }
  }
}

// BlendPixel for the modes the compositor's common form takes: kClear,
// kSrc, kDst, kSrcOver (their FastBlend rules and PMSrcOver).
SKC_HD uint32_t BlendPixelCommon(uint32_t dst, uint32_t src, uint32_t mode) {
  switch (mode) {
    case 0: return 0;
    case 1: return src;
    case 2: return dst;
    default: {
      const uint32_t a = GetA(src);
      if (a == 0) return dst;
      if (a == 255) return src;
      return PMSrcOver(src, dst);
    }
  }
}

// PorterDuff out of line: the compositor's loop keeps only the common modes'
// code (its registers are budgeted for the residency it runs at).
SKC_HDN uint32_t PorterDuffOutOfLine(uint32_t src, uint32_t dst, uint32_t mode) {
  return PorterDuff(src, dst, mode);
}

// SWRenderTarget::BlendPixel (sw_render_target.cc:12-35): the FastBlend
// shortcuts (:89-141), else PorterDuffBlend; returns the new destination.
SKC_HD uint32_t BlendPixel(uint32_t dst, uint32_t src, uint32_t mode) {
  switch (mode) {
    case 0: return 0;        // kClear
    case 1: return src;      // kSrc
    case 2: return dst;      // kDst
    case 3: {                // kSrcOver
      const uint32_t a = GetA(src);
      if (a == 0) return dst;
      if (a == 255) return src;
      return PMSrcOver(src, dst);
    }
    case 4:                  // kDstOver
      if (GetA(dst) == 255) return dst;
      break;
    case 6: {                // kDstIn
      const uint32_t a = GetA(src);
      if (a == 255) return dst;
      if (a == 0) return 0;
      break;
    }
    case 8: {                // kDstOut
      const uint32_t a = GetA(src);
      if (a == 0) return dst;
      if (a == 255) return 0;
      break;
    }
    default:
      break;
  }
  return PorterDuffOutOfLine(src, dst, mode);
}

// One pixel of MaskFilterOnFilter's combine (mask_filter.cc:61-100) for
// BlurStyle kSolid (2), kOuter (3), kInner (4): raw = the unblurred draw,
// blur = its StackBlur (both ARGB); returns the filtered pixel.
SKC_HD uint32_t BlurStylePixel(uint32_t style, uint32_t raw, uint32_t blur) {
  const uint32_t raw_a = GetA(raw), blur_a = GetA(blur);
  if (style == 2) return raw_a > 0 ? raw : blur;
  if (style == 3) return (raw_a > 0 && raw_a >= blur_a) ? 0u : blur;
  if (style == 4) {
    if (raw_a == 0) return 0;
    const float a_factor = 1.f / 255.f;
    return AlphaMulQ(blur, (uint32_t)(a_factor * raw_a * blur_a));
  }
  return blur;
}

// PMColorToColor (color_priv.cc:20-104): channel * (255 << 24) / a, rounded,
// as UnPreMultiply's scale table holds it (entry a = round(255 * 2^24 / a)).
SKC_HD uint32_t UnpremulScale(uint32_t a) {
  return a == 0 ? 0u : (uint32_t)(((255ull << 24) + a / 2) / a);
}
SKC_HD uint32_t PMColorToColor(uint32_t c) {
  const uint32_t a = GetA(c), s = UnpremulScale(a);
  auto ch = [&](uint32_t v) { return (s * v + (1u << 23)) >> 24; };  // uint32 arithmetic
  return ARGB(a, ch(GetR(c)), ch(GetG(c)), ch(GetB(c)));
}

// ColorFilter::FilterColor (color_filter.cc:56-186) of a premultiplied
// colour.  tables: [0, 256) linear->sRGB, [256, 512) sRGB->linear;
// matrices: int16 terms (row_major * 255, truncated), 4 rows of 5.
SKC_HDN uint32_t FilterColorOutOfLine(uint32_t cf_type, uint32_t cf_mode, uint32_t cf_pm,
                                      uint32_t cf_index, uint32_t c, const uint8_t* tables,
                                      const int16_t* matrices);
SKC_HD uint32_t FilterColor(const Brush& b, uint32_t c, const uint8_t* tables,
                            const int16_t* matrices) {
  return FilterColorOutOfLine(b.cf_type, b.cf_mode, b.cf_pm, b.cf_index, c, tables, matrices);
}
SKC_HDN uint32_t FilterColorOutOfLine(uint32_t cf_type, uint32_t cf_mode, uint32_t cf_pm,
                                      uint32_t cf_index, uint32_t c, const uint8_t* tables,
                                      const int16_t* matrices) {
  Brush b;
  b.cf_type = cf_type;
  b.cf_mode = cf_mode;
  b.cf_pm = cf_pm;
  b.cf_index = cf_index;
  switch (b.cf_type) {
    case 1:  // BlendColorFilter: PorterDuffBlend(filter colour, c, mode)
      return PorterDuff(b.cf_pm, c, b.cf_mode);
    case 2: {  // MatrixColorFilter
      const uint32_t u = PMColorToColor(c);
      const int32_t v[4] = {(int32_t)GetR(u), (int32_t)GetG(u), (int32_t)GetB(u), (int32_t)GetA(u)};
      const int16_t* m = matrices + b.cf_index;
      uint32_t o[4];
      for (int i = 0; i < 4; ++i) {
        const int32_t mul = v[0] * m[5 * i] + v[1] * m[5 * i + 1] + v[2] * m[5 * i + 2] +
                            v[3] * m[5 * i + 3];
        o[i] = (uint32_t)min_(max_(mul / 255 + m[5 * i + 4], 0), 255);
      }
      return ColorToPMColor(ARGB(o[3], o[0], o[1], o[2]));
    }
    case 3:
    case 4: {  // SRGBGammaColorFilter
      const uint32_t u = PMColorToColor(c);
      const uint8_t* t = tables + (b.cf_type == 3 ? 0 : 256);
      return ColorToPMColor(ARGB(GetA(u), t[GetR(u)], t[GetG(u)], t[GetB(u)]));
    }
    default:
      return c;
  }
}

SKC_HD float RemapFloatTile(float t, uint32_t tile) {  // sw_span_brush.cc:21-32
  if (tile == 0) {
    t = min_(max_(t, 0.0f), 1.0f);
  } else if (tile == 1) {
    t = t - floor_(t);
  } else if (tile == 2) {
    // float - 2 * std::floor(float * 0.5) - 1 evaluates in double
    float t1 = t - 1;
    float t2 = (float)((double)t1 - 2.0 * floor((double)t1 * 0.5) - 1.0);
    t = fabs_(t2);
  }
  return t;
}

// GradientColorBrush::LerpColor (sw_span_brush.cc:232-296) -> premul ARGB
SKC_HD uint32_t GradientColor(const Brush& b, float current, const float4* colors,
                              const float* offsets) {
  const float kNZ = 1.0f / (1 << 12);
  if (fabs_(current) <= kNZ) {
    current = 0.0f;
  } else if (fabs_(current - 1.0f) <= kNZ) {
    current = 1.0f;
  }
  if (b.tile == 3 && (current < 0.0f || current >= 1.0f)) return 0;
  current = RemapFloatTile(current, b.tile);
  int color_count = (int)b.stop_count;
  int stop_count = b.has_offsets ? color_count : 0;
  const float4* c = colors + b.stop0;
  const float* o = offsets + b.stop0;
  float4 out;
  if (stop_count > 0 && current <= o[0]) {
    out = c[0];
  } else {
    float step = 1.f / (color_count - 1);
    int i = 0, si = 0, ei = 1;
    float start = 0.f, end = 0.f;
    for (i = 0; i < color_count - 1; i++) {
      if (stop_count > 0) {
        start = o[i];
        end = o[i + 1];
      } else {
        start = step * i;
        end = step * (i + 1);
      }
      if (current >= start && current <= end) {
        si = i;
        ei = i + 1;
        break;
      }
    }
    if (i == color_count - 1 && color_count > 0) {
      out = c[color_count - 1];
    } else {
      float total = end - start;
      float value = current - start;
      float mix = 0.5f;
      if (total > 0) mix = value / total;
      float om = 1 - mix;
      out.x = c[si].x * om + c[ei].x * mix;
      out.y = c[si].y * om + c[ei].y * mix;
      out.z = c[si].z * om + c[ei].z * mix;
      out.w = c[si].w * om + c[ei].w * mix;
    }
  }
  return ColorToPMColor(Color4fToColor(out.x, out.y, out.z, out.w));
}

// SweepGradientColorBrush::CalculateColor's parameter (sw_span_brush.cc:
// 336-349) at the mapped point: the angle of (-y, -x) as a float
// (std::atan2 on floats), then (angle / 2pi + 0.5 + bias) * scale in double
// (0.5 is a double literal there).  The float angle is the double atan2
// rounded to float.
SKC_HD float SweepT(const Brush& b, float mx, float my) {
  const float angle = (float)atan2d_((double)-my, (double)-mx);
  const float k1Over2Pi = 0.1591549430918f;
  return (float)(((double)(angle * k1Over2Pi) + 0.5 + (double)b.bias) * (double)b.scale);
}

// ConicalGradientColorBrush::CalculateConical (sw_span_brush.cc:441-507):
// false when the pixel is transparent, else the gradient parameter.
SKC_HD bool ConicalT(const ConicalParams& c, int x, int y, float* t_out) {
  if (c.mode == 0 || c.mode == 2) return false;
  const float sx = x + 0.5f, sy = y + 0.5f;
  const float px = sx * c.d2l[0] + sy * c.d2l[1] + c.d2l[2];
  const float py = sx * c.d2l[3] + sy * c.d2l[4] + c.d2l[5];
  float t;
  if (c.mode == 1) {
    const float qx = (px - c.c0x) * c.scale, qy = (py - c.c0y) * c.scale;
    t = sqrt_(qx * qx + qy * qy) * c.scale_sign - c.bias;
  } else {
    const float qx = px * c.t[0] + py * c.t[1] + c.t[2];
    const float qy = px * c.t[3] + py * c.t[4] + c.t[5];
    if (c.mode == 3) {
      t = c.r2 - qy * qy;
      if (t < 0.0f) return false;
      t = (float)((double)qx + sqrtd_((double)t));  // sqrt of a float here is ::sqrt(double)
    } else {
      float xt = -1.f;
      if (fabs_(c.r1 - 1.f) < 1.0f / (1 << 12)) {
        xt = (qx * qx + qy * qy) / 2;
      } else {
        const float m = c.r1_square - 1.f;
        const float delta = m * qy * qy + c.r1_square * qx * qx;
        if (c.r1 > 1.f) {
          xt = (sqrt_(delta) - qx) / m;
        } else if (delta > 0) {
          const float xt1 = (sqrt_(delta) - qx) / m;
          const float xt2 = (-sqrt_(delta) - qx) / m;
          xt = 1.f - c.f < 0 ? (xt2 < xt1 ? xt2 : xt1) : (xt1 < xt2 ? xt2 : xt1);
        }
      }
      if (xt < 0) return false;
      t = c.f + (1.f - c.f) * xt;
      if (c.swap01) t = (float)(1.0 - (double)t);
    }
  }
  *t_out = t;
  return true;
}

// CalculateColor of the pass's brush at pixel (x, y), premultiplied ARGB.
// roundtrip[v] = Color4fToColor(Color4fFromColor(v)) per channel, the
// PixmapBrush sampler's colour round trip (bitmap_sampler.cc:21-29,93-107).
// The sweep and two-point conical brushes out of line (they are rare, and
// their code would crowd the compositor's loop): the brush's gradient
// fields by value.
SKC_HDN uint32_t OtherGradientColor(uint32_t kind, uint32_t tile, uint32_t stop_count,
                                    uint32_t has_offsets, uint32_t stop0, float bias, float scale,
                                    uint32_t conical, float mx, float my, int x, int y,
                                    const float4* colors, const float* offsets,
                                    const ConicalParams* conicals) {
  Brush g;
  g.tile = tile;
  g.stop_count = stop_count;
  g.has_offsets = has_offsets;
  g.stop0 = stop0;
  g.bias = bias;
  g.scale = scale;
  float t;
  if (kind == 5) {
    if (!ConicalT(conicals[conical], x, y, &t)) return 0;
  } else {
    t = SweepT(g, mx, my);
  }
  return GradientColor(g, t, colors, offsets);
}

// Image shader mode word: tile modes, bilinear filter, unpremultiplied pixels.
SKC_HD uint32_t ImageMode(uint32_t tile_x, uint32_t tile_y, bool linear, bool unpremul) {
  return tile_x | (tile_y << 4) | ((linear ? 1u : 0u) << 8) | ((unpremul ? 1u : 0u) << 12);
}

// RemapFloatTile (bitmap_sampler.cc:12-23): 0 clamp, 1 repeat, 2 mirror
// (its floor in double), 3 decal (left as is).
SKC_HD float RemapTile(float t, uint32_t mode) {
  if (mode == 0) return t < 0.0f ? 0.0f : (1.0f < t ? 1.0f : t);
  if (mode == 1) return t - floorf(t);
  if (mode == 2) {
    const float t1 = t - 1;
    const float t2 = (float)((double)t1 - 2 * floor((double)t1 * 0.5) - 1);
    return fabsf(t2);
  }
  return t;
}

// glm::clamp<uint32_t>(v, 0, n - 1) of a float coordinate
// (BitmapSampler::SampleXY, bitmap_sampler.cc:26-34).  The float converts
// to uint32_t as x86-64 compilers do it (through a 64-bit signed integer),
// so a coordinate of -1 wraps to the last column, as the reference's own
// build computes it.
SKC_HD uint32_t SampleIndex(float v, uint32_t n) {
  const uint32_t u = (uint32_t)(long long)v;
  return u < n - 1 ? u : n - 1;
}

SKC_HD float4 SampleTexel(const uint8_t* img, uint32_t w, uint32_t h, float x, float y) {
  const uint8_t* px = img + ((size_t)SampleIndex(y, h) * w + SampleIndex(x, w)) * 4;
  // Color4fFromColor (color.cc:44-51)
  return make_float4(px[0] / 255.f, px[1] / 255.f, px[2] / 255.f, px[3] / 255.f);
}

// PixmapBrush::CalculateColor (sw_span_brush.cc:568-579) through
// BitmapSampler::GetColor (bitmap_sampler.cc:36-108), at unit coordinates
// (u, v).
SKC_HDN uint32_t ImageShaderColor(float u, float v, uint32_t mode, uint32_t w, uint32_t h,
                                  const uint8_t* img) {
  const uint32_t tx = mode & 15, ty = (mode >> 4) & 15;
  if ((tx == 3 && (u < 0.0f || u >= 1.0f)) || (ty == 3 && (v < 0.0f || v >= 1.0f))) return 0;
  u = RemapTile(u, tx);
  v = RemapTile(v, ty);
  const float fw = (float)w, fh = (float)h;
  float4 c;
  if (mode & 256) {  // SampleUnitLinear
    const float x = u * fw, y = v * fh;
    float i0 = floorf(x - 0.5f), j0 = floorf(y - 0.5f);
    if (tx == 1) i0 = i0 - fw * floorf(i0 / fw);  // glm::mod
    if (ty == 1) j0 = j0 - fh * floorf(j0 / fh);
    float i1 = i0 + 1.0f, j1 = j0 + 1.0f;
    if (tx == 1) i1 = i1 - fw * floorf(i1 / fw);
    if (ty == 1) j1 = j1 - fh * floorf(j1 / fh);
    const float xa = x - 0.5f, yb = y - 0.5f;
    const float a = xa - floorf(xa), b = yb - floorf(yb);  // glm::fract
    const float4 t00 = SampleTexel(img, w, h, i0, j0), t10 = SampleTexel(img, w, h, i1, j0);
    const float4 t01 = SampleTexel(img, w, h, i0, j1), t11 = SampleTexel(img, w, h, i1, j1);
    const float w00 = (1 - a) * (1 - b), w10 = a * (1 - b), w01 = (1 - a) * b, w11 = a * b;
    c.x = w00 * t00.x + w10 * t10.x + w01 * t01.x + w11 * t11.x;
    c.y = w00 * t00.y + w10 * t10.y + w01 * t01.y + w11 * t11.y;
    c.z = w00 * t00.z + w10 * t10.z + w01 * t01.z + w11 * t11.z;
    c.w = w00 * t00.w + w10 * t10.w + w01 * t01.w + w11 * t11.w;
  } else {  // SampleUnitNearest
    c = SampleTexel(img, w, h, u * fw, v * fh);
  }
  // Color4fToColor, then ColorToPMColor for unpremultiplied pixels
  const uint32_t col =
      ARGB(ChannelToByte(c.w), ChannelToByte(c.x), ChannelToByte(c.y), ChannelToByte(c.z));
  return (mode & 4096) ? ColorToPMColor(col) : col;
}

// BrushColor for the solid, linear, radial and image brushes.
SKC_HD uint32_t BrushColorCommon(const Brush& b, int x, int y, const float4* colors,
                                 const float* offsets, const uint8_t* images,
                                 const uint8_t* roundtrip) {
  if (b.kind == 0) return b.solid;
  float sx = x + 0.5f, sy = y + 0.5f;
  float mx = sx * b.m[0] + sy * b.m[1] + b.m[2];
  float my = sx * b.m[3] + sy * b.m[4] + b.m[5];
  if (b.kind == 1) return GradientColor(b, mx, colors, offsets);
  if (b.kind == 2) return GradientColor(b, sqrt_(mx * mx + my * my), colors, offsets);
  if (mx < 0.0f || mx >= 1.0f || my < 0.0f || my >= 1.0f) return 0;
  uint32_t ix = (uint32_t)(mx * (float)b.img_w), iy = (uint32_t)(my * (float)b.img_h);
  ix = min_(ix, b.img_w - 1);
  iy = min_(iy, b.img_h - 1);
  const uint8_t* px = images + b.img_off + ((size_t)iy * b.img_w + ix) * 4;
  return ARGB(roundtrip[px[3]], roundtrip[px[0]], roundtrip[px[1]], roundtrip[px[2]]);
}

SKC_HD uint32_t BrushColor(const Brush& b, int x, int y, const float4* colors, const float* offsets,
                           const uint8_t* images, const uint8_t* roundtrip,
                           const ConicalParams* conicals) {
  if (b.kind == 0) return b.solid;
  float sx = x + 0.5f, sy = y + 0.5f;
  float mx = sx * b.m[0] + sy * b.m[1] + b.m[2];
  float my = sx * b.m[3] + sy * b.m[4] + b.m[5];
  if (b.kind == 1) return GradientColor(b, mx, colors, offsets);
  if (b.kind == 2) return GradientColor(b, sqrt_(mx * mx + my * my), colors, offsets);
  if (b.kind == 6) return ImageShaderColor(mx, my, b.tile, b.img_w, b.img_h, images + b.img_off);
  if (b.kind >= 4)
    return OtherGradientColor(b.kind, b.tile, b.stop_count, b.has_offsets, b.stop0, b.bias, b.scale,
                              b.conical, mx, my, x, y, colors, offsets, conicals);
  // image brush, decal tiling, nearest sampling
  if (mx < 0.0f || mx >= 1.0f || my < 0.0f || my >= 1.0f) return 0;
  uint32_t ix = (uint32_t)(mx * (float)b.img_w), iy = (uint32_t)(my * (float)b.img_h);
  ix = min_(ix, b.img_w - 1);
  iy = min_(iy, b.img_h - 1);
  const uint8_t* px = images + b.img_off + ((size_t)iy * b.img_w + ix) * 4;
  return ARGB(roundtrip[px[3]], roundtrip[px[0]], roundtrip[px[1]], roundtrip[px[2]]);
}

}  // namespace skc
