/* Defines boundary tables as a problem's global.hpp does and prints the ones
 * the library sees (no GPU needed). */
#include <stdio.h>

int dnxs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int dnys[8] = {+1, +1, -1, +1, +1, +1, -1, +1};

int mlau_boundary_tables(int *dnx, int *dny, int *dnz);

int main(void)
{
    int x[8], y[8], z[8];
    mlau_boundary_tables(x, y, z);
    for (int v = 0; v < 8; v++) printf("%d %d %d\n", x[v], y[v], z[v]);
    return 0;
}
