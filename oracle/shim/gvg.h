/* the reference includes gvg.h, which it does not ship; nothing in the
   compiled routines needs its contents */
