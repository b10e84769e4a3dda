/* Headless stand-in for <GL/gl.h>, used only to compile the reference's
 * draw* methods (never executed by the oracle harness). Every call is a
 * no-op expression; no graphics library is loaded. */
#ifndef ESF_ORACLE_SHIM_GL_H
#define ESF_ORACLE_SHIM_GL_H
typedef float GLfloat;
typedef double GLdouble;
typedef int GLint;
typedef unsigned int GLenum;
typedef unsigned char GLboolean;
#define GL_LINES 1
#define GL_POINTS 0
#define GL_TRIANGLES 4
#define glBegin(...) ((void)0)
#define glEnd(...) ((void)0)
#define glColor3d(...) ((void)0)
#define glColor3f(...) ((void)0)
#define glColor4f(...) ((void)0)
#define glNormal3d(...) ((void)0)
#define glNormal3f(...) ((void)0)
#define glPointSize(...) ((void)0)
#define glPopMatrix(...) ((void)0)
#define glPushMatrix(...) ((void)0)
#define glScaled(...) ((void)0)
#define glTranslated(...) ((void)0)
#define glTranslatef(...) ((void)0)
#define glVertex3d(...) ((void)0)
#define glVertex3f(...) ((void)0)
#define glutSolidCube(...) ((void)0)
#define glutWireCube(...) ((void)0)
#endif
