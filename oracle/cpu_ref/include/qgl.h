// Compile-time stand-ins for the gl* names the reference's draw methods
// mention, so that the translation units holding its solver compile
// headless.  They do nothing; the draw methods are never called and no
// graphics library is involved.  Test infrastructure.
#pragma once

enum {
    GL_LINES = 1, GL_POINTS, GL_QUADS, GL_TRIANGLE_FAN, GL_LINE, GL_FILL, GL_FRONT_AND_BACK, GL_BLEND
};
inline void glBegin(int) {}
inline void glEnd() {}
inline void glColor3f(float, float, float) {}
inline void glColor4f(float, float, float, float) {}
inline void glVertex2f(float, float) {}
inline void glVertex2d(double, double) {}
inline void glEnable(int) {}
inline void glDisable(int) {}
inline void glLineWidth(float) {}
inline void glPointSize(float) {}
inline void glPolygonMode(int, int) {}
inline void glPushMatrix() {}
inline void glPopMatrix() {}
inline void glRotatef(float, float, float, float) {}
inline void glScalef(float, float, float) {}
inline void glTranslatef(float, float, float) {}
