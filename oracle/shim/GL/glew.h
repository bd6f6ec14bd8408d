/* Test infrastructure (oracle only): link-time stand-ins that let the reference's
 * OpenCloth_Implicit/OpenCloth_Implicit/main.cpp and
 * OpenCloth_CoRotated_Linear_FEM/OpenCloth_CoRotated_Linear_FEM/main.cpp compile headless.  Every GL, GLU,
 * GLUT and WGL call expands to a no-op expression; no graphics stack is involved.
 * Only ref_harness.cpp includes this directory. */
#ifndef OC_SHIM_GLEW_H
#define OC_SHIM_GLEW_H
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>

typedef unsigned short GLushort;
typedef int GLint;
typedef unsigned int GLenum;
typedef float GLfloat;
typedef double GLdouble;

/* Win32 bits used by the reference's FPS counter (main.cpp:90, :115-116, :473-476, :624). */
#define MAX_PATH 260
typedef union { long long QuadPart; } LARGE_INTEGER;
#define QueryPerformanceFrequency(...) (0)
#define QueryPerformanceCounter(...) (0)
#define sprintf_s(buf, ...) snprintf((buf), sizeof(buf), __VA_ARGS__)

/* GL / GLU: arguments are discarded unevaluated. */
#define glewInit(...) (0)
#define glEnable(...) (0)
#define glClear(...) (0)
#define glLoadIdentity(...) (0)
#define glTranslatef(...) (0)
#define glRotatef(...) (0)
#define glGetDoublev(...) (0)
#define glGetIntegerv(...) (0)
#define glColor3f(...) (0)
#define glVertex3f(...) (0)
#define glBegin(...) (0)
#define glEnd(...) (0)
#define glPushMatrix(...) (0)
#define glPopMatrix(...) (0)
#define glMultMatrixf(...) (0)
#define glPolygonMode(...) (0)
#define glPointSize(...) (0)
#define glViewport(...) (0)
#define glMatrixMode(...) (0)
#define glReadPixels(...) (0)
#define gluPerspective(...) (0)
#define gluUnProject(...) (0)
#endif
