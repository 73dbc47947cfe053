#pragma once
// Generated by oracle/gen_mc_tables.py -- do not edit by hand.
// Per Marching Cubes case (bit i set <=> corner i >= iso), the cell's
// contours packed as: nibbles 0-3 = contour sizes, nibbles 4-15 = the
// intersected cell edges of all contours back to back (0xF = unused).
// Same contour/edge order as the reference's polygon table
// (MarchingCubes/VisualDMC/src/DMC/DualMarchingCubes.cpp:564), packed as
// its Contour class does (D/CellIntersection.h:28-137).  Ambiguous cases
// do not read this table.
#define MDMC_CONTOUR_WORDS \
    0xffffffffffff0000ULL, 0xfffffffff3800003ULL, 0xfffffffff9100003ULL, 0xffffffff91380004ULL, \
    0xfffffffff2b30003ULL, 0xffffffff802b0004ULL, 0xffffffb320910033ULL, 0xfffffff8912b0005ULL, \
    0xfffffffffa210003ULL, 0xffffffa213800033ULL, 0xffffffff09a20004ULL, 0xfffffff9a2380005ULL, \
    0xffffffffb31a0004ULL, 0xfffffffb801a0005ULL, 0xfffffffab3090005ULL, 0xffffffffab890004ULL, \
    0xfffffffff8740003ULL, 0xffffffff74030004ULL, 0xffffff7489100033ULL, 0xfffffff374910005ULL, \
    0xffffff2b37480033ULL, 0xfffffff02b740005ULL, 0xfffb327481090333ULL, 0xffffff912b740006ULL, \
    0xffffff748a210033ULL, 0xfffffa2103740034ULL, 0xfffff74809a20034ULL, 0xffffff3749a20006ULL, \
    0xfffff487b31a0034ULL, 0xffffff7401ab0006ULL, 0xffffab3098740053ULL, 0xfffffff9ab740005ULL, \
    0xfffffffff4590003ULL, 0xffffff3804590033ULL, 0xffffffff10450004ULL, 0xfffffff138450005ULL, \
    0xffffffb324590033ULL, 0xfffff594802b0034ULL, 0xfffffb3210450034ULL, 0xffffffb845120006ULL, \
    0xffffff459a210033ULL, 0xfff594a218030333ULL, 0xfffffff045a20005ULL, 0xffffff3845a20006ULL, \
    0xfffff4591ab30034ULL, 0xffff1ab805940053ULL, 0xffffffab30450006ULL, 0xfffffffab8450005ULL, \
    0xffffffff59870004ULL, 0xfffffff759030005ULL, 0xfffffff510870005ULL, 0xffffffff37510004ULL, \
    0xfffff2b387590034ULL, 0xffffff02b7590006ULL, 0xffff87510b320053ULL, 0xfffffff7512b0005ULL, \
    0xfffff21a59870034ULL, 0xffff0375921a0053ULL, 0xffffff75a2080006ULL, 0xfffffff375a20005ULL, \
    0xffffb31a87590044ULL, 0xfffff901ab750007ULL, 0xfffff30875ab0007ULL, 0xffffffff75ab0004ULL, \
    0xfffffffffb670003ULL, 0xffffff67b8030033ULL, 0xffffff67b9100033ULL, 0xfffff67b38910034ULL, \
    0xffffffff67320004ULL, 0xfffffff267800005ULL, 0xfffff91032670034ULL, 0xffffff7891260006ULL, \
    0xffffff7b621a0033ULL, 0xfff7b6803a210333ULL, 0xfffff7b6a2090034ULL, 0xffff389a27b60053ULL, \
    0xfffffff31a670005ULL, 0xffffff801a670006ULL, 0xffffff9a67300006ULL, 0xfffffff89a670005ULL, \
    0xffffffffb6480004ULL, 0xfffffff403b60005ULL, 0xfffff10948b60034ULL, 0xffffff13b6490006ULL, \
    0xfffffff648320005ULL, 0xffffffff26400004ULL, 0xffff648320910053ULL, 0xfffffff264910005ULL, \
    0xfffff1a2b6480034ULL, 0xffffb6403a210053ULL, 0xffff9a20648b0044ULL, 0xfffff23b649a0007ULL, \
    0xffffffa648310006ULL, 0xfffffff6401a0005ULL, 0xfffff8309a640007ULL, 0xffffffff649a0004ULL, \
    0xffffffb675940033ULL, 0xfff67b5943800333ULL, 0xfffffb6745100034ULL, 0xffff4513867b0053ULL, \
    0xfffff94567320034ULL, 0xffff267804590053ULL, 0xffff045173260044ULL, 0xfffff78451260007ULL, \
    0xfffb6721a4590333ULL, 0x594380a217b63333ULL, 0xffffa2045b670053ULL, 0xfff67b5a23840036ULL, \
    0xffff6731a4590053ULL, 0xfff4597801a60036ULL, 0xfffff5a673040007ULL, 0xffffff845a670006ULL, \
    0xfffffff8b6590005ULL, 0xffffff5903b60006ULL, 0xffffff65108b0006ULL, 0xfffffff513b60005ULL, \
    0xffffff3265980006ULL, 0xfffffff026590005ULL, 0xfffff08326510007ULL, 0xffffffff26510004ULL, \
    0xffff8b659a210053ULL, 0xfffa2165903b0036ULL, 0xfffff65a208b0007ULL, 0xffffff5a23b60006ULL, \
    0xfffffa6598310007ULL, 0xffffff65901a0006ULL, 0xffffffa658300033ULL, 0xfffffffff65a0003ULL, \
    0xfffffffff56a0003ULL, 0xffffff6a53800033ULL, 0xffffff6a51090033ULL, 0xfffff6a591380034ULL, \
    0xffffff56ab320033ULL, 0xfffff56a2b800034ULL, 0xfff6a5b329100333ULL, 0xffff2b8916a50053ULL, \
    0xffffffff21560004ULL, 0xfffff80321560034ULL, 0xfffffff209560005ULL, 0xffffff6238950006ULL, \
    0xfffffff156b30005ULL, 0xffffff156b800006ULL, 0xffffff0956b30006ULL, 0xfffffffb89560005ULL, \
    0xffffff8746a50033ULL, 0xfffffa5674030034ULL, 0xfff7486a50910333ULL, 0xffff3749156a0053ULL, \
    0xfff56a4872b30333ULL, 0xffff02b746a50053ULL, 0x6a5b328749103333ULL, 0xfff6a5b749120036ULL, \
    0xfffff87456210034ULL, 0xffff740356210044ULL, 0xffff562097480053ULL, 0xfffff49562370007ULL, \
    0xffff156b37480053ULL, 0xfffff6b740150007ULL, 0xfff7486b30950036ULL, 0xffffffb749560006ULL, \
    0xffffffff6a940004ULL, 0xfffff380946a0034ULL, 0xfffffff46a100005ULL, 0xffffff46a1380006ULL, \
    0xfffff32b6a940034ULL, 0xffff6a942b800044ULL, 0xffff46a102b30053ULL, 0xfffffa12b8460007ULL, \
    0xfffffff621940005ULL, 0xffff946218030053ULL, 0xffffffff46200004ULL, 0xfffffff462380005ULL, \
    0xffffffb319460006ULL, 0xfffff01946b80007ULL, 0xfffffff046b30005ULL, 0xffffffffb8460004ULL, \
    0xfffffff9876a0005ULL, 0xffffff6a90370006ULL, 0xffffff10876a0006ULL, 0xfffffff1376a0005ULL, \
    0xffff9876ab320053ULL, 0xfffffb76a9020007ULL, 0xfffb3276a1080036ULL, 0xffffff76a12b0006ULL, \
    0xffffff9876210006ULL, 0xfffff19037620007ULL, 0xfffffff620870005ULL, 0xffffffff62370004ULL, \
    0xfffff76b31980007ULL, 0xffffff76b1900033ULL, 0xffffff6b30870006ULL, 0xfffffffff6b70003ULL, \
    0xffffffff7ba50004ULL, 0xfffff0387ba50034ULL, 0xfffff091a57b0034ULL, 0xffff1389ba570044ULL, \
    0xfffffff732a50005ULL, 0xffffffa578020006ULL, 0xffff732a51090053ULL, 0xfffff12a57890007ULL, \
    0xfffffff57b210005ULL, 0xffff57b213800053ULL, 0xffffffb209570006ULL, 0xfffffb2389570007ULL, \
    0xffffffff57310004ULL, 0xfffffff157800005ULL, 0xfffffff573090005ULL, 0xffffffff57890004ULL, \
    0xfffffffba5480005ULL, 0xffffff3ba5400006ULL, 0xffffba5489100053ULL, 0xfffff54913ba0007ULL, \
    0xffffff4832a50006ULL, 0xfffffff402a50005ULL, 0xfff91054832a0036ULL, 0xffffff4912a50006ULL, \
    0xffffff48b2150006ULL, 0xfffff3b215400007ULL, 0xfffff9548b200007ULL, 0xffffff3b25490033ULL, \
    0xfffffff315480005ULL, 0xffffffff15400004ULL, 0xffffff3095480006ULL, 0xfffffffff5490003ULL, \
    0xfffffffa947b0005ULL, 0xffff7ba943800053ULL, 0xffffff047ba10006ULL, 0xfffff847ba130007ULL, \
    0xffffff4732a90006ULL, 0xfffff47802a90007ULL, 0xfffff2a104730007ULL, 0xffffff4782a10033ULL, \
    0xffffff21947b0006ULL, 0xfff380b219470036ULL, 0xfffffff2047b0005ULL, 0xffffff23847b0006ULL, \
    0xfffffff731940005ULL, 0xffffff7801940006ULL, 0xffffffff73040004ULL, 0xfffffffff7840003ULL, \
    0xffffffff8ba90004ULL, 0xfffffffba9030005ULL, 0xfffffff8ba100005ULL, 0xffffffffba130004ULL, \
    0xfffffffa98320005ULL, 0xffffffff02a90004ULL, 0xffffffa108320006ULL, 0xfffffffff2a10003ULL, \
    0xfffffff98b210005ULL, 0xffffffb219030006ULL, 0xffffffff8b200004ULL, 0xfffffffffb230003ULL, \
    0xffffffff98310004ULL, 0xfffffffff1900003ULL, 0xfffffffff8300003ULL, 0xffffffffffff0000ULL

namespace mdmc {
// Lives in global memory; kernels stage it in shared memory (lanes index it
// with divergent cases, which would serialise a __constant__ read).
__device__ const unsigned long long kContourTable[256] = {MDMC_CONTOUR_WORDS};
static const unsigned long long kContourTableHost[256] = {MDMC_CONTOUR_WORDS};
}  // namespace mdmc
