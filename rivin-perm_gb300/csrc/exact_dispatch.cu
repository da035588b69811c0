// Dispatch over the compiled (order, group size) pairs of the exact kernel.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_0(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_1(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_2(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_3(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_4(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_5(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_6(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_7(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);

static bool dispatch(int N, int G, const ExactArgs *args, int blocks,
                     cudaStream_t stream, cudaError_t *err, int *occ) {
    if (exact_dispatch_0(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_1(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_2(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_3(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_4(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_5(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_6(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_7(N, G, args, blocks, stream, err, occ)) return true;
    return false;
}

bool exact_compiled(int N, int G) {
    if (N < 2 || N > 48 || G < 1 || G > 7) return false;
    switch (N * 8 + G) {
    case 17:
    case 18:
    case 25:
    case 26:
    case 27:
    case 33:
    case 34:
    case 35:
    case 36:
    case 41:
    case 42:
    case 43:
    case 44:
    case 49:
    case 50:
    case 51:
    case 52:
    case 57:
    case 58:
    case 59:
    case 60:
    case 65:
    case 66:
    case 67:
    case 68:
    case 73:
    case 74:
    case 75:
    case 76:
    case 81:
    case 82:
    case 83:
    case 84:
    case 89:
    case 90:
    case 91:
    case 92:
    case 97:
    case 98:
    case 99:
    case 100:
    case 105:
    case 106:
    case 107:
    case 108:
    case 113:
    case 114:
    case 115:
    case 116:
    case 121:
    case 122:
    case 123:
    case 124:
    case 129:
    case 130:
    case 131:
    case 132:
    case 138:
    case 139:
    case 140:
    case 146:
    case 147:
    case 148:
    case 154:
    case 155:
    case 156:
    case 162:
    case 163:
    case 164:
    case 170:
    case 171:
    case 172:
    case 178:
    case 179:
    case 180:
    case 186:
    case 187:
    case 188:
    case 194:
    case 195:
    case 196:
    case 197:
    case 198:
    case 202:
    case 203:
    case 204:
    case 205:
    case 206:
    case 210:
    case 211:
    case 212:
    case 213:
    case 214:
    case 218:
    case 219:
    case 220:
    case 221:
    case 222:
    case 226:
    case 227:
    case 228:
    case 229:
    case 230:
    case 234:
    case 235:
    case 236:
    case 237:
    case 238:
    case 242:
    case 243:
    case 244:
    case 245:
    case 246:
    case 250:
    case 251:
    case 252:
    case 253:
    case 254:
    case 258:
    case 259:
    case 260:
    case 261:
    case 262:
    case 267:
    case 268:
    case 269:
    case 270:
    case 275:
    case 276:
    case 277:
    case 278:
    case 283:
    case 284:
    case 285:
    case 286:
    case 291:
    case 292:
    case 293:
    case 294:
    case 299:
    case 300:
    case 301:
    case 302:
    case 307:
    case 308:
    case 309:
    case 310:
    case 315:
    case 316:
    case 317:
    case 318:
    case 323:
    case 324:
    case 325:
    case 326:
    case 331:
    case 332:
    case 333:
    case 334:
    case 339:
    case 340:
    case 341:
    case 342:
    case 347:
    case 348:
    case 349:
    case 350:
    case 355:
    case 356:
    case 357:
    case 358:
    case 363:
    case 364:
    case 365:
    case 366:
    case 371:
    case 372:
    case 373:
    case 374:
    case 379:
    case 380:
    case 381:
    case 382:
    case 387:
    case 388:
    case 389:
    case 390:
        return true;
    default:
        return false;
    }
}

cudaError_t launch_exact_any(int N, int G, const ExactArgs &args, int blocks,
                             cudaStream_t stream) {
    cudaError_t err = cudaErrorInvalidValue;
    if (!dispatch(N, G, &args, blocks, stream, &err, nullptr)) return cudaErrorInvalidValue;
    return err;
}

int occupancy_exact_any(int N, int G) {
    cudaError_t err = cudaSuccess;
    int occ = 1;
    if (!dispatch(N, G, nullptr, 0, nullptr, &err, &occ)) return 1;
    return occ;
}

}  // namespace pg
