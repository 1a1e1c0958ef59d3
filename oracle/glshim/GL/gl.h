/* Typedef-only stand-in for <GL/gl.h>.
 *
 * The reference's libtxc_dxtn header includes <GL/gl.h> only for the GL scalar
 * typedefs and the four S3TC format enums.  No GL library is linked or needed
 * to compile the encoder, so this header supplies exactly those names (values
 * from the public EXT_texture_compression_s3tc registry entry). */
#ifndef S2TC_ORACLE_GLSHIM_H
#define S2TC_ORACLE_GLSHIM_H
typedef int GLint;
typedef unsigned char GLubyte;
typedef unsigned int GLenum;
typedef void GLvoid;
#define GL_COMPRESSED_RGB_S3TC_DXT1_EXT  0x83F0
#define GL_COMPRESSED_RGBA_S3TC_DXT1_EXT 0x83F1
#define GL_COMPRESSED_RGBA_S3TC_DXT3_EXT 0x83F2
#define GL_COMPRESSED_RGBA_S3TC_DXT5_EXT 0x83F3
#endif
