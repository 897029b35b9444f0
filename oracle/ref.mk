# Builds the REFERENCE's own CPU ray caster into oracle/_ref/ (test infrastructure only):
# Helios core (Context, global) and the CollisionDetection plug-in, compiled unchanged from
# the reference tree together with the zlib, libpng, libjpeg and pugixml sources it vendors,
# plus ref_raycast.cpp (this directory), the C entry points the tests call.
#
#   make -f ref.mk REF=/root/reference -j8
#
# No reference build system runs.  Two configuration headers the vendored libraries ship
# are copied, unchanged, under the names their sources include: zlib's zconf.h.included
# (the stock zconf.h) as zconf.h and libjpeg's jconfig.txt as jconfig.h.
REF ?= /root/reference
OUT := _ref
CC ?= gcc
CXX ?= g++
CFLAGS := -O2 -fPIC -w
CXXFLAGS := -O2 -std=c++17 -fPIC -fopenmp -ffp-contract=off -w
LIB := $(REF)/core/lib
INC := -I$(OUT)/include -I$(REF)/core/include -I$(LIB)/pugixml -I$(LIB)/zlib -I$(LIB)/libpng \
       -I$(LIB)/libjpeg-9a -I$(LIB)/tinyexr -I$(REF)/plugins/collisiondetection/include

ZLIB := adler32 compress crc32 deflate gzclose gzlib gzread gzwrite infback inffast inflate inftrees trees uncompr zutil
PNG := png pngerror pngget pngmem pngpread pngread pngrio pngrtran pngrutil pngset pngtrans pngwio pngwrite pngwtran pngwutil
JPEG := jmemnobs jaricom jcapimin jcapistd jcarith jccoefct jccolor jcdctmgr jchuff jcinit jcmainct jcmarker \
        jcmaster jcomapi jcparam jcprepct jcsample jctrans jdapimin jdapistd jdarith jdatadst jdatasrc jdcoefct \
        jdcolor jddctmgr jdhuff jdinput jdmainct jdmarker jdmaster jdmerge jdpostct jdsample jdtrans jerror \
        jfdctflt jfdctfst jfdctint jidctflt jidctfst jidctint jquant1 jquant2 jutils jmemmgr
CORE := Context Context_data Context_fileIO Context_object Context_primitive global exif_writer
CD := CollisionDetection CollisionDetection_RayTracing CollisionDetection_Slicing

OBJ := $(ZLIB:%=$(OUT)/obj/zlib/%.o) $(PNG:%=$(OUT)/obj/png/%.o) $(JPEG:%=$(OUT)/obj/jpeg/%.o) \
       $(OUT)/obj/pugixml.o $(CORE:%=$(OUT)/obj/core/%.o) $(CD:%=$(OUT)/obj/cd/%.o) $(OUT)/obj/ref_raycast.o
HDR := $(OUT)/include/zconf.h $(OUT)/include/jconfig.h

$(OUT)/libref_raycast.so: $(OBJ)
	$(CXX) -shared -fopenmp $^ -o $@

$(OUT)/include/zconf.h: $(LIB)/zlib/zconf.h.included
	@mkdir -p $(dir $@)
	cp $< $@
$(OUT)/include/jconfig.h: $(LIB)/libjpeg-9a/jconfig.txt
	@mkdir -p $(dir $@)
	cp $< $@

$(OUT)/obj/zlib/%.o: $(LIB)/zlib/%.c $(HDR)
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) $(INC) -c $< -o $@
$(OUT)/obj/png/%.o: $(LIB)/libpng/%.c $(HDR)
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) -DPNG_ARM_NEON_OPT=0 $(INC) -c $< -o $@
$(OUT)/obj/jpeg/%.o: $(LIB)/libjpeg-9a/%.c $(HDR)
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) $(INC) -c $< -o $@
$(OUT)/obj/pugixml.o: $(LIB)/pugixml/pugixml.cpp $(HDR)
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@
$(OUT)/obj/core/%.o: $(REF)/core/src/%.cpp $(HDR)
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@
$(OUT)/obj/cd/%.o: $(REF)/plugins/collisiondetection/src/%.cpp $(HDR)
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@
$(OUT)/obj/ref_raycast.o: ref_raycast.cpp $(HDR)
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

clean:
	rm -rf $(OUT)
.PHONY: clean
