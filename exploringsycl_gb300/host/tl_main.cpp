/* tl_main.cpp -- command-line entry of the TeaLeaf driver (TeaLeaf/main.c). */
extern "C" int tl_main(int argc, char** argv);

int main(int argc, char** argv) { return tl_main(argc, argv); }
