/* Headless stand-in for GLEW used only to compile the reference's CUDA step without OpenGL
 * (test infrastructure; oracle/build_ref.sh).  Declares the GL names that the reference's
 * buffer templates mention; none of them is ever called by the headless driver.  The
 * reference's debug-string sink (a Win32 call) is routed to the driver, which reads the
 * solver loop counts from it. */
#pragma once
typedef unsigned int GLenum;
typedef unsigned int GLuint;
typedef int GLint;
typedef int GLsizei;
typedef unsigned char GLboolean;
typedef long GLsizeiptr;
typedef long GLintptr;
typedef float GLfloat;
#define GL_DYNAMIC_DRAW 0x88E8
#define GL_STATIC_DRAW 0x88E4
#define GL_ARRAY_BUFFER 0x8892
extern "C" void mps_ref_debug_sink(const char* msg);
inline void OutputDebugStringA(const char* msg) { mps_ref_debug_sink(msg); }
template <class... A> inline void glCreateBuffers(A...) {}
template <class... A> inline void glDeleteBuffers(A...) {}
template <class... A> inline GLboolean glIsBuffer(A...) { return 0; }
template <class... A> inline void glNamedBufferData(A...) {}
template <class... A> inline void glNamedBufferSubData(A...) {}
template <class... A> inline void glNamedCopyBufferSubDataEXT(A...) {}
