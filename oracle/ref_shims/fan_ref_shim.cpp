// Stubs that let the reference's helical/rebin/src/tracing.cpp link on its
// own (its utility.cpp needs Boost, which is not installed).  The two helper
// functions restate utility.cpp:33-37 (sqr, get_img_addr); the globals are the
// ones main.h declares extern and tracing.cpp reads.  Test infrastructure only.
int NX = 0, NY = 0;
double vx = 1.0, vy = 1.0;

double sqr(double x) { return x * x; }
double get_img_addr(double x, double y) { return x * NY + y; }

void forward_proj(double sx, double sy, double dx, double dy, int *ind, double *wgt, int &numb);

extern "C" int fanref_trace(int n, double pixel_mm, double sx, double sy, double dx, double dy,
                            int *ind, double *wgt) {
    NX = NY = n;
    vx = vy = pixel_mm;
    int numb = 0;
    forward_proj(sx, sy, dx, dy, ind, wgt, numb);
    return numb;
}
