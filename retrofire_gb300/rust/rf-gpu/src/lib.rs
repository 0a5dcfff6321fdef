//! rf-gpu: retrofire's `render()` with a GPU render target.
//!
//! The reference renders on the CPU through
//!
//! ```text
//! pub fn render(prims, verts, shader: &Shd, uniform: Uni,
//!               to_screen: Mat4<Ndc, Screen>, target: &mut impl Target,
//!               ctx: &Context)                        core/src/render.rs:134-147
//! ```
//!
//! This crate keeps that call shape and the reference's own types
//! (`Tri<usize>`, `Vertex3<A>`, `ProjMat3`, `Mat4<Ndc, Screen>`, `Context`,
//! `Stats`, `Buf2`) and runs the path on librfgpu (rf-gpu-sys): a caller
//! swaps `&mut Framebuf<..>` for `&mut GpuFramebuf` and its closure shader
//! for the `GpuShader` that computes the same thing.  Results equal the CPU
//! path's bit for bit (colour within one LSB for `GouraudSrgb`).
//!
//! The reference's `Target::rasterize` is called per scanline
//! (target.rs:18-31); a GPU target cannot be driven that way, so
//! `GpuFramebuf` is not an `impl Target`: `render` here takes it directly,
//! and the per-scanline work happens on the device.
//!
//! Unverified: neither this machine nor the GPU machine has a Rust toolchain,
//! so this crate has not been compiled.  The C ABI underneath is tested
//! through its Python binding.
#![allow(clippy::too_many_arguments)]

use core::cell::RefCell;
use core::cmp::Ordering;
use core::ptr;

use rf_gpu_sys as sys;
use retrofire_core::geom::{Tri, Vertex3};
use retrofire_core::math::{Color3f, Color4, Mat4, ProjMat3};
use retrofire_core::render::{
    ctx::{DepthSort, FaceCull},
    Context, Model, Ndc, Screen, Stats, TexCoord,
};
use retrofire_core::util::buf::Buf2;

/// A non-zero rf_status with the library's message.
#[derive(Debug, Clone, Copy, PartialEq, Eq)]
pub struct Error(pub i32);

fn check(code: sys::rf_status) -> Result<(), Error> {
    if code == sys::RF_OK { Ok(()) } else { Err(Error(code)) }
}

/// One rf_ctx: a CUDA stream and the handles created on it (one per host
/// thread, as the reference's `Context` is not `Sync`).
pub struct Device {
    ctx: *mut sys::rf_ctx,
}

impl Device {
    /// A device context on the current CUDA device with a private stream.
    pub fn new() -> Result<Self, Error> {
        let mut ctx = ptr::null_mut();
        check(unsafe { sys::rf_ctx_create(ptr::null_mut(), &mut ctx) })?;
        Ok(Self { ctx })
    }
    /// Waits for all queued work.
    pub fn sync(&self) -> Result<(), Error> {
        check(unsafe { sys::rf_ctx_sync(self.ctx) })
    }
    pub fn raw(&self) -> *mut sys::rf_ctx {
        self.ctx
    }
}

impl Drop for Device {
    fn drop(&mut self) {
        unsafe { sys::rf_ctx_destroy(self.ctx) };
    }
}

/// The vertex attribute types the fixed shader family reads, flattened to
/// f32s in the order the reference's `Vary` impls interpolate them.
pub trait GpuAttrib: Copy {
    const N: u32;
    fn push(&self, out: &mut Vec<f32>);
}
impl GpuAttrib for () {
    const N: u32 = 0;
    fn push(&self, _: &mut Vec<f32>) {}
}
impl GpuAttrib for Color3f {
    const N: u32 = 3;
    fn push(&self, out: &mut Vec<f32>) {
        out.extend_from_slice(&self.0);
    }
}
impl GpuAttrib for TexCoord {
    const N: u32 = 2;
    fn push(&self, out: &mut Vec<f32>) {
        out.push(self.x());
        out.push(self.y());
    }
}
impl GpuAttrib for (Color3f, TexCoord) {
    const N: u32 = 5;
    fn push(&self, out: &mut Vec<f32>) {
        self.0.push(out);
        self.1.push(out);
    }
}

/// A mesh resident on the device: `prims` and `verts` of a render() call,
/// uploaded once (render.rs borrows them per call instead).
pub struct GpuMesh<'d> {
    dev: &'d Device,
    handle: sys::rf_mesh,
    nattr: u32,
}

impl<'d> GpuMesh<'d> {
    pub fn new<A: GpuAttrib>(dev: &'d Device, prims: &[Tri<usize>], verts: &[Vertex3<A>]) -> Result<Self, Error> {
        let mut v = Vec::with_capacity(verts.len() * (3 + A::N as usize));
        for vx in verts {
            v.push(vx.pos.x());
            v.push(vx.pos.y());
            v.push(vx.pos.z());
            vx.attrib.push(&mut v);
        }
        let mut idx = Vec::with_capacity(prims.len() * 3);
        for t in prims {
            for &i in &t.0 {
                // An index past u32 would also be past the vertices: the
                // library refuses it like `vs[i]` panics (prim.rs:17-19).
                idx.push(u32::try_from(i).unwrap_or(u32::MAX));
            }
        }
        let mut h = 0;
        check(unsafe {
            sys::rf_mesh_upload(dev.ctx, v.as_ptr(), verts.len() as u32, 3, A::N, idx.as_ptr(),
                                prims.len() as u32, &mut h)
        })?;
        Ok(Self { dev, handle: h, nattr: A::N })
    }
}

impl Drop for GpuMesh<'_> {
    fn drop(&mut self) {
        unsafe { sys::rf_mesh_destroy(self.dev.ctx, self.handle) };
    }
}

/// A texture resident on the device (`Texture<Buf2<Color4>>`, tex.rs:33-37).
pub struct GpuTexture<'d> {
    dev: &'d Device,
    handle: sys::rf_texture,
}

impl<'d> GpuTexture<'d> {
    pub fn new(dev: &'d Device, texels: &Buf2<Color4>) -> Result<Self, Error> {
        let data: Vec<u32> = texels.data().iter().map(|c| u32::from_le_bytes(c.0)).collect();
        let mut h = 0;
        check(unsafe {
            sys::rf_texture_upload(dev.ctx, data.as_ptr(), texels.width(), texels.height(), &mut h)
        })?;
        Ok(Self { dev, handle: h })
    }
}

impl Drop for GpuTexture<'_> {
    fn drop(&mut self) {
        unsafe { sys::rf_texture_destroy(self.dev.ctx, self.handle) };
    }
}

/// The samplers of tex.rs:218-357.
#[derive(Copy, Clone, Debug)]
pub enum Sampler {
    RepeatPot,
    Clamp,
    Once,
}

/// The fixed shader family that replaces the reference's closure shaders
/// (shader.rs:31-76).  Each variant computes what the closure pair in its
/// comment computes; the vertex side is always
/// `|v, mvp| vertex(mvp.apply(&v.pos), v.attrib)`.
#[derive(Copy, Clone)]
pub enum GpuShader<'t> {
    /// `|_: Frag<()>| color` (benches/fill.rs:21-34), attrib `()`.
    Flat(Color4),
    /// `|f: Frag<Color3f>| f.var.to_color4()` (color.rs:253-263).
    Gouraud,
    /// `|f: Frag<Color3f>| f.var.to_srgb().to_color4()` (hello_tri.rs:12-20).
    GouraudSrgb,
    /// `|f: Frag<TexCoord>| sampler.sample(&tex, f.var)`.
    Textured(&'t GpuTexture<'t>, Sampler),
    /// `|f: Frag<(Color3f, TexCoord)>|
    ///      (sampler.sample(&tex, f.var.1).to_rgb().to_color3f() * f.var.0).to_color4()`.
    TexGouraud(&'t GpuTexture<'t>, Sampler),
}

impl GpuShader<'_> {
    fn kind_and_attrs(&self) -> (i32, u32) {
        match self {
            GpuShader::Flat(_) => (sys::RF_SHADER_FLAT, 0),
            GpuShader::Gouraud => (sys::RF_SHADER_GOURAUD, 3),
            GpuShader::GouraudSrgb => (sys::RF_SHADER_GOURAUD_SRGB, 3),
            GpuShader::Textured(..) => (sys::RF_SHADER_TEXTURED, 2),
            GpuShader::TexGouraud(..) => (sys::RF_SHADER_TEX_GOURAUD, 5),
        }
    }
    fn uniforms(&self, mvp: &ProjMat3<Model>) -> sys::rf_uniforms {
        let mut u = sys::rf_uniforms { mvp: [0.0; 16], flat_rgba: 0, sampler: 0, texture: 0 };
        for (r, row) in mvp.0.iter().enumerate() {
            u.mvp[4 * r..4 * r + 4].copy_from_slice(row);
        }
        let samp = |s: &Sampler| match s {
            Sampler::RepeatPot => sys::RF_SAMPLER_REPEAT_POT,
            Sampler::Clamp => sys::RF_SAMPLER_CLAMP,
            Sampler::Once => sys::RF_SAMPLER_ONCE,
        };
        match self {
            GpuShader::Flat(c) => u.flat_rgba = u32::from_le_bytes(c.0),
            GpuShader::Textured(t, s) | GpuShader::TexGouraud(t, s) => {
                u.texture = t.handle;
                u.sampler = samp(s);
            }
            _ => {}
        }
        u
    }
}

/// Pixel formats of the colour buffer (`IntoPixel<u32, F>`, pixfmt.rs:76-103).
#[derive(Copy, Clone, Debug)]
pub enum PixFmt {
    Argb8888,
    Xrgb8888,
    Rgba8888,
    Bgra8888,
}

/// The GPU counterpart of `Framebuf<Colorbuf<Buf2<u32>, F>, Buf2<f32>>`
/// (target.rs:35-44), or of a colour-only `Colorbuf` without depth.
pub struct GpuFramebuf<'d> {
    dev: &'d Device,
    handle: sys::rf_target,
    w: u32,
    h: u32,
    depth: bool,
}

impl<'d> GpuFramebuf<'d> {
    pub fn new(dev: &'d Device, w: u32, h: u32, fmt: PixFmt, depth: bool) -> Result<Self, Error> {
        let f = match fmt {
            PixFmt::Argb8888 => sys::RF_ARGB8888,
            PixFmt::Xrgb8888 => sys::RF_XRGB8888,
            PixFmt::Rgba8888 => sys::RF_RGBA8888,
            PixFmt::Bgra8888 => sys::RF_BGRA8888,
        };
        let mut h_ = 0;
        check(unsafe { sys::rf_target_create(dev.ctx, w, h, f, depth as i32, &mut h_) })?;
        Ok(Self { dev, handle: h_, w, h, depth })
    }

    /// `Frame::clear` (front/src/lib.rs:103-120) with the context's clear
    /// values: colour <- into_pixel(color_clear), depth <- 1 / depth_clear.
    pub fn clear(&mut self, ctx: &Context) -> Result<(), Error> {
        let c = ctx.color_clear.map(|c| u32::from_le_bytes(c.0));
        let z = ctx.depth_clear;
        check(unsafe {
            sys::rf_target_clear(
                self.dev.ctx,
                self.handle,
                c.as_ref().map_or(ptr::null(), |c| c as *const u32),
                z.as_ref().map_or(ptr::null(), |z| z as *const f32),
            )
        })
    }

    /// Copies the target into host buffers of the same dimensions.
    pub fn read(&self, color: &mut Buf2<u32>, depth: Option<&mut Buf2<f32>>) -> Result<(), Error> {
        assert!(color.width() == self.w && color.height() == self.h);
        let dp = match depth {
            Some(d) if self.depth => {
                assert!(d.width() == self.w && d.height() == self.h);
                d.data_mut().as_mut_ptr()
            }
            _ => ptr::null_mut(),
        };
        check(unsafe { sys::rf_target_read(self.dev.ctx, self.handle, color.data_mut().as_mut_ptr(), dp) })
    }
}

impl Drop for GpuFramebuf<'_> {
    fn drop(&mut self) {
        unsafe { sys::rf_target_destroy(self.dev.ctx, self.handle) };
    }
}

fn flags(ctx: &Context) -> sys::rf_context_flags {
    sys::rf_context_flags {
        depth_test: match ctx.depth_test {
            None => sys::RF_DEPTH_NONE,
            Some(Ordering::Less) => sys::RF_DEPTH_LESS,
            Some(Ordering::Equal) => sys::RF_DEPTH_EQUAL,
            Some(Ordering::Greater) => sys::RF_DEPTH_GREATER,
        },
        color_write: ctx.color_write as i32,
        depth_write: ctx.depth_write as i32,
        face_cull: match ctx.face_cull {
            None => sys::RF_CULL_NONE,
            Some(FaceCull::Back) => sys::RF_CULL_BACK,
            Some(FaceCull::Front) => sys::RF_CULL_FRONT,
        },
        depth_sort: match ctx.depth_sort {
            None => sys::RF_SORT_NONE,
            Some(DepthSort::FrontToBack) => sys::RF_SORT_FRONT_TO_BACK,
            Some(DepthSort::BackToFront) => sys::RF_SORT_BACK_TO_FRONT,
        },
    }
}

fn add_stats(acc: &RefCell<Stats>, s: &sys::rf_stats) {
    let mut st = acc.borrow_mut();
    st.calls += s.calls as f32;
    st.prims.i += s.prims_i as usize;
    st.prims.o += s.prims_o as usize;
    st.verts.i += s.verts_i as usize;
    st.verts.o += s.verts_o as usize;
    st.frags.i += s.frags_i as usize;
    st.frags.o += s.frags_o as usize;
    st.objs.i += s.objs_i as usize;
    st.objs.o += s.objs_o as usize;
}

/// `render(prims, verts, shader, uniform, to_screen, target, ctx)` with the
/// primitives and vertices already on the device; adds this call's stats
/// into `ctx.stats` as render.rs:206 does.
pub fn render(
    mesh: &GpuMesh,
    shader: &GpuShader,
    uniform: &ProjMat3<Model>,
    to_screen: &Mat4<Ndc, Screen>,
    target: &mut GpuFramebuf,
    ctx: &Context,
) -> Result<(), Error> {
    let (kind, nattr) = shader.kind_and_attrs();
    if nattr != mesh.nattr {
        return Err(Error(sys::RF_ERR_BAD_ARG));
    }
    let u = shader.uniforms(uniform);
    let mut vp = [0.0f32; 16];
    for (r, row) in to_screen.0.iter().enumerate() {
        vp[4 * r..4 * r + 4].copy_from_slice(row);
    }
    let fl = flags(ctx);
    let mut st = sys::rf_stats::default();
    check(unsafe {
        sys::rf_render(mesh.dev.ctx, mesh.handle, kind, &u, vp.as_ptr(), target.handle, &fl, &mut st)
    })?;
    add_stats(&ctx.stats, &st);
    Ok(())
}

/// The reference's exact call shape: uploads `prims` and `verts` for this
/// call only (like render() borrowing its slices), then renders.
pub fn render_slices<A: GpuAttrib>(
    prims: &[Tri<usize>],
    verts: &[Vertex3<A>],
    shader: &GpuShader,
    uniform: &ProjMat3<Model>,
    to_screen: &Mat4<Ndc, Screen>,
    target: &mut GpuFramebuf,
    ctx: &Context,
) -> Result<(), Error> {
    let mesh = GpuMesh::new(target.dev, prims, verts)?;
    render(&mesh, shader, uniform, to_screen, target, ctx)
}
